// server.cpp — continuous-batching render server.
//
// Requests (a scene + a shot: camera, resolution, spp) arrive at any time.
// `slots` worker threads each own a context (CUDA stream + wavefront
// buffers), so the work of several requests overlaps on the device.  A slot
// keeps an active set of requests on the same scene and renders them as one
// multi-shot wavefront per chunk of frames; after each chunk, finished
// requests leave the set and pending requests of that scene join it (as long
// as the memory budget admits their films), so new work enters as soon as
// slots and memory free up.  Requests whose footprint can never fit, or that
// arrive while the pending queue is full, are rejected.
//
// Scenes: added ones are built at once and stay resident; registered ones
// are built by the worker that admits their first request (charged to the
// budget with an estimate until the build reports its size) and dropped,
// least recently used first, when an admission needs memory and no request
// uses them.
//
// Denoised requests render the two halves of their frames into two films;
// when both are done the slot's denoiser blends the denoise of all samples
// with their plain average (asuna_denoise_blended) into the result image.
//
// Each path's sample stream depends only on (pixel, frame, shot seed) and
// the denoiser is deterministic, so a request renders the same result alone
// or in any mix (tested).
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

#include <cuda_runtime.h>

#include "../../include/asuna_denoise.h"
#include "../../include/asuna_rt.h"
#include "common.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  uint64_t id = 0;
  uint32_t scene = 0;
  uint32_t flags = 0;
  asuna_shot shot{};
  double arrival = 0, start = -1, finish = -1;
  uint32_t frames[2] = {0, 0};  // frames of each part (a denoised request has two)
  uint32_t done[2] = {0, 0};    // frames rendered per part
  int status = ASUNA_OK;
  bool charged = false;  // admitted: `bytes` are counted in the server's memory
  uint64_t bytes = 0;    // films + denoised image
  asuna_film* film[2] = {nullptr, nullptr};
  float* denoised = nullptr;  // device RGBA, denoised requests
  asuna_ctx* filmCtx = nullptr;
  std::mutex io;  // a read of the films and their release exclude each other
  bool denoise() const { return (flags & ASUNA_REQUEST_DENOISE) != 0; }
  int parts() const { return denoise() ? 2 : 1; }
  bool complete() const { return done[0] >= frames[0] && done[1] >= frames[1]; }
};

struct SceneEntry {
  const asuna_scene_desc* desc = nullptr;  // registered: built on demand
  asuna_scene* dev = nullptr;
  uint64_t bytes = 0;     // charged to the budget (the estimate while building)
  uint64_t estimate = 0;
  int users = 0;          // admitted requests not yet finished
  bool building = false;
  double lastUse = 0;
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
  std::deque<SceneEntry> scenes;  // (a deque: entries keep their addresses as scenes are added)
  std::vector<asuna_ctx*> ctxs;
  // Reads of finished films: the slots' streams may be capturing the next
  // request's graph, so copies out go on a stream of the server's own.
  cudaStream_t readStream = nullptr;
  std::vector<asuna_denoiser*> denoisers;  // one per slot, or none
  std::vector<std::thread> workers;
  uint64_t memUsed = 0;  // films held + scenes
  uint64_t nextId = 1;
  int inFlight = 0;
  bool stop = false;
  uint64_t rejected = 0, admitted = 0, samples = 0, built = 0, evicted = 0, denoised = 0;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

uint64_t filmBytes(const asuna_shot& s) { return uint64_t(s.width) * s.height * 16ull * 9ull; }

uint64_t requestBytes(const asuna_shot& s, bool denoise) {
  return denoise ? 2 * filmBytes(s) + uint64_t(s.width) * s.height * 16ull : filmBytes(s);
}

// Device bytes a scene will take: nodes (about one 64-byte node per
// triangle at most), leaf triangles, shading vertices and indices,
// instances, materials, lights, the environment map and its tables,
// textures.
uint64_t sceneEstimate(const asuna_scene_desc* d) {
  uint64_t tris = 0, verts = 0, texels = 0;
  for (uint32_t m = 0; m < d->num_meshes; ++m) {
    tris += d->meshes[m].num_triangles;
    verts += d->meshes[m].num_vertices;
  }
  for (uint32_t t = 0; t < d->num_textures; ++t) texels += uint64_t(d->textures[t].width) * d->textures[t].height;
  const uint64_t env = d->envmap.rgba ? uint64_t(d->envmap.width) * d->envmap.height * 32 : 32;
  return tris * (64 + 48 + 16) + verts * 32 + uint64_t(d->num_instances) * (128 + 128) +
         uint64_t(d->num_materials) * 96 + uint64_t(d->num_lights) * 80 + env + texels * 16 + (1u << 20);
}

// Drops idle registered scenes, least recently used first, until `need`
// more bytes fit or none is left to drop (caller holds the lock; returns
// the scenes to destroy outside it).
void evictFor(asuna_server* S, uint64_t need, uint32_t keep, std::vector<asuna_scene*>& drop) {
  while (S->memUsed + need > S->opts.memory_budget) {
    int victim = -1;
    for (size_t i = 0; i < S->scenes.size(); ++i) {
      const SceneEntry& e = S->scenes[i];
      if (i == keep || !e.desc || !e.dev || e.building || e.users > 0) continue;
      if (victim < 0 || e.lastUse < S->scenes[size_t(victim)].lastUse) victim = int(i);
    }
    if (victim < 0) return;
    SceneEntry& e = S->scenes[size_t(victim)];
    S->memUsed -= e.bytes;
    drop.push_back(e.dev);
    e.dev = nullptr;
    e.bytes = 0;
    S->evicted++;
  }
}

// Takes pending requests of `scene` (any scene if scene < 0) that the memory
// budget admits, up to `room`, oldest first.  A request whose registered
// scene is not resident also needs the scene's estimate (its builder is
// whoever admits it: `*build` receives the scene).  Caller holds the lock.
void admit(asuna_server* S, int scene, size_t room, std::vector<std::shared_ptr<Req>>& out, int* build,
           std::vector<asuna_scene*>& drop) {
  for (auto it = S->pending.begin(); it != S->pending.end() && room > 0;) {
    auto& r = *it;
    if (scene >= 0 && int(r->scene) != scene) {
      ++it;
      continue;
    }
    SceneEntry& e = S->scenes[r->scene];
    if (e.building) {  // another slot is building it: wait
      if (scene < 0) break;
      ++it;
      continue;
    }
    const bool needBuild = !e.dev;
    const uint64_t need = r->bytes + (needBuild ? e.estimate : 0);
    if (S->memUsed + need > S->opts.memory_budget) evictFor(S, need, r->scene, drop);
    if (S->memUsed + need > S->opts.memory_budget) {
      if (scene < 0) break;  // keep arrival order for new sets
      ++it;
      continue;
    }
    if (needBuild) {
      e.building = true;
      e.bytes = e.estimate;
      *build = int(r->scene);
    }
    S->memUsed += need;
    r->charged = true;
    e.users++;
    e.lastUse = S->now();
    r->start = S->now();
    out.push_back(r);
    if (scene < 0) scene = int(r->scene);
    it = S->pending.erase(it);
    --room;
  }
}

// Film images of the guides a denoised request needs (albedo, normal).
bool guideImages(const asuna_shot& s, int* albedo, int* normal) {
  *albedo = s.state.diffuse_out_channel >= 0 ? 1 + s.state.diffuse_out_channel : -1;
  *normal = s.state.normal_out_channel >= 0 ? 1 + s.state.normal_out_channel : -1;
  return *albedo > 0 && *normal > 0;
}

void finishRequest(asuna_server* S, const std::shared_ptr<Req>& r, double t) {
  r->finish = t;
  SceneEntry& e = S->scenes[r->scene];
  e.users--;
  e.lastUse = t;
  S->finished.push_back(r);
}

void worker(asuna_server* S, int slot) {
  asuna_ctx* ctx = S->ctxs[slot];
  std::vector<std::shared_ptr<Req>> active;
  const size_t maxSet = std::max(1u, S->opts.max_batch);
  for (;;) {
    int build = -1;
    const asuna_scene_desc* buildDesc = nullptr;
    std::vector<asuna_scene*> drop;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->stop && !active.empty()) {
        // shutting down: abandon the active set
        for (auto& r : active) {
          r->status = ASUNA_ERR_TIMEOUT;
          finishRequest(S, r, S->now());
        }
        active.clear();
        S->inFlight--;
        return;
      }
      if (active.empty()) {
        S->cv.wait(lk, [&] { return S->stop || !S->pending.empty(); });
        if (S->stop && S->pending.empty()) return;
        admit(S, -1, maxSet, active, &build, drop);
        if (active.empty()) {
          lk.unlock();
          for (auto* sc : drop) asuna_scene_destroy(sc);
          lk.lock();
          // nothing fits right now: wait for memory to be released
          S->cv.wait_for(lk, std::chrono::milliseconds(2));
          continue;
        }
        S->inFlight++;
      } else {
        admit(S, int(active[0]->scene), maxSet - active.size(), active, &build, drop);
      }
      if (build >= 0) buildDesc = S->scenes[size_t(build)].desc;
    }
    for (auto* sc : drop) asuna_scene_destroy(sc);
    const uint32_t sid = active[0]->scene;
    if (build >= 0) {
      // the scene's device build, at admission of its first request
      asuna_scene* dev = nullptr;
      int rc = asuna_scene_create(ctx, buildDesc, &dev);
      asuna_scene_stats st{};
      if (rc == ASUNA_OK) asuna_scene_get_stats(dev, &st);
      std::lock_guard<std::mutex> lk(S->mu);
      SceneEntry& e = S->scenes[size_t(build)];
      S->memUsed -= e.bytes;
      e.building = false;
      if (rc == ASUNA_OK) {
        e.dev = dev;
        e.bytes = st.device_bytes;
        S->memUsed += e.bytes;
        S->built++;
      } else {
        e.bytes = 0;
        for (auto& r : active)
          if (r->status == ASUNA_OK) r->status = rc;
      }
    }
    // films for newly admitted requests
    for (auto& r : active) {
      if (r->status != ASUNA_OK || r->film[0]) continue;
      for (int k = 0; k < r->parts() && r->status == ASUNA_OK; ++k)
        if (asuna_film_create(ctx, r->shot.width, r->shot.height, &r->film[k]) != ASUNA_OK) r->status = ASUNA_ERR_OOM;
      if (r->status == ASUNA_OK && r->denoise() &&
          cudaMalloc(reinterpret_cast<void**>(&r->denoised), size_t(r->shot.width) * r->shot.height * 16) !=
              cudaSuccess) {
        cudaGetLastError();
        r->status = ASUNA_ERR_OOM;
      }
      r->filmCtx = ctx;
    }
    // one chunk: every active request (part) advances by up to frames_per_chunk frames
    std::vector<asuna_shot> shots;
    std::vector<asuna_film*> films;
    std::vector<std::pair<Req*, int>> owners;
    for (auto& r : active) {
      if (r->status != ASUNA_OK) continue;
      for (int k = 0; k < r->parts(); ++k) {
        if (r->done[k] >= r->frames[k]) continue;
        asuna_shot s = r->shot;
        s.frame0 = r->shot.frame0 + (k ? r->frames[0] : 0) + r->done[k];
        s.frames = std::min(S->opts.frames_per_chunk, r->frames[k] - r->done[k]);
        shots.push_back(s);
        films.push_back(r->film[k]);
        owners.push_back({r.get(), k});
      }
    }
    int rc = ASUNA_OK;
    if (!shots.empty()) {
      asuna_scene* dev = nullptr;
      {
        std::lock_guard<std::mutex> lk(S->mu);
        dev = S->scenes[sid].dev;
      }
      rc = dev ? asuna_render_batch(ctx, dev, shots.data(), films.data(), uint32_t(shots.size()), nullptr)
               : ASUNA_ERR_INVALID;
      if (rc == ASUNA_OK) rc = asuna_ctx_sync(ctx);
    }
    for (size_t k = 0; k < owners.size(); ++k) {
      Req* r = owners[k].first;
      if (rc != ASUNA_OK)
        r->status = rc;
      else
        r->done[owners[k].second] += shots[k].frames;
    }
    // denoise the requests whose halves are both rendered
    uint64_t denoisedNow = 0;
    for (auto& r : active) {
      if (r->status != ASUNA_OK || !r->denoise() || !r->complete() || r->finish >= 0) continue;
      int albedo, normal;
      guideImages(r->shot, &albedo, &normal);
      double err = 0, errPlain = 0, w = 0;
      asuna_denoiser* d = S->denoisers.empty() ? nullptr : S->denoisers[slot];
      int drc = d ? asuna_denoise_blended(ctx, d, r->film[0], r->film[1], albedo, normal, r->denoised, &err,
                                          &errPlain, &w)
                  : ASUNA_ERR_INVALID;
      if (drc == ASUNA_OK) drc = asuna_ctx_sync(ctx);
      if (drc != ASUNA_OK) r->status = drc;
      else ++denoisedNow;
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      const double t = S->now();
      S->denoised += denoisedNow;
      for (size_t k = 0; k < owners.size(); ++k)
        if (rc == ASUNA_OK) S->samples += uint64_t(shots[k].frames) * shots[k].width * shots[k].height;
      for (auto it = active.begin(); it != active.end();) {
        auto& r = *it;
        if (r->status != ASUNA_OK || r->complete()) {
          finishRequest(S, r, t);
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

void freeRequest(Req& r) {
  for (auto*& f : r.film) {
    if (f) asuna_film_destroy(f);
    f = nullptr;
  }
  if (r.denoised) cudaFree(r.denoised);
  r.denoised = nullptr;
}

int addScene(asuna_server* S, const asuna_scene_desc* desc, bool registerOnly, uint32_t* scene_id) {
  asuna::clearError();
  if (!S || !desc || !scene_id) return asuna::fail(ASUNA_ERR_INVALID, "null argument");
  SceneEntry e;
  if (registerOnly) {
    int rc = asuna_scene_validate(desc);
    if (rc) return rc;
    e.desc = desc;
    e.estimate = sceneEstimate(desc);
    if (e.estimate > S->opts.memory_budget)
      return asuna::fail(ASUNA_ERR_OOM, "scene of about %llu bytes exceeds the server memory budget",
                         (unsigned long long)e.estimate);
  } else {
    int rc = asuna_scene_create(S->ctxs[0], desc, &e.dev);
    if (rc) return rc;
    asuna_scene_stats st;
    asuna_scene_get_stats(e.dev, &st);
    e.bytes = st.device_bytes;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (!registerOnly) {
    if (S->memUsed + e.bytes > S->opts.memory_budget) {
      asuna_scene_destroy(e.dev);
      return asuna::fail(ASUNA_ERR_OOM, "scene of %llu bytes exceeds the server memory budget",
                         (unsigned long long)e.bytes);
    }
    S->memUsed += e.bytes;
  }
  S->scenes.push_back(e);
  *scene_id = uint32_t(S->scenes.size() - 1);
  return ASUNA_OK;
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
  if (cudaSetDevice(opts->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&S->readStream, cudaStreamNonBlocking) != cudaSuccess) {
    for (auto* x : S->ctxs) asuna_ctx_destroy(x);
    delete S;
    return asuna::fail(ASUNA_ERR_CUDA, "asuna_server_create: stream creation failed");
  }
  for (uint32_t i = 0; i < opts->slots; ++i) S->workers.emplace_back(worker, S, int(i));
  *out = S;
  return ASUNA_OK;
}

int asuna_server_add_scene(asuna_server* S, const asuna_scene_desc* desc, uint32_t* scene_id) {
  return addScene(S, desc, false, scene_id);
}

int asuna_server_register_scene(asuna_server* S, const asuna_scene_desc* desc, uint32_t* scene_id) {
  return addScene(S, desc, true, scene_id);
}

int asuna_server_set_denoiser(asuna_server* S, const asuna_denoiser_opts* opts, const float* params, uint64_t n) {
  asuna::clearError();
  if (!S || !opts || !params) return asuna::fail(ASUNA_ERR_INVALID, "asuna_server_set_denoiser: null argument");
  std::vector<asuna_denoiser*> ds;
  for (asuna_ctx* c : S->ctxs) {
    asuna_denoiser* d = nullptr;
    int rc = asuna_denoiser_create(c, opts, &d);
    if (rc == ASUNA_OK) rc = asuna_denoiser_set_params(d, params, n);
    if (rc != ASUNA_OK) {
      if (d) asuna_denoiser_destroy(d);
      for (auto* x : ds) asuna_denoiser_destroy(x);
      return rc;
    }
    ds.push_back(d);
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (!S->denoisers.empty() || S->inFlight > 0) {
    for (auto* x : ds) asuna_denoiser_destroy(x);
    return asuna::fail(ASUNA_ERR_INVALID, "set the denoiser once, before submitting requests");
  }
  S->denoisers = ds;
  return ASUNA_OK;
}

int asuna_server_submit(asuna_server* S, const asuna_request* req, uint64_t* id) {
  asuna::clearError();
  if (!S || !req || !id) return asuna::fail(ASUNA_ERR_INVALID, "null argument");
  auto r = std::make_shared<Req>();
  r->scene = req->scene;
  r->flags = req->flags;
  r->shot = req->shot;
  r->frames[0] = r->denoise() ? (req->shot.frames + 1) / 2 : req->shot.frames;
  r->frames[1] = r->denoise() ? req->shot.frames - r->frames[0] : 0;
  r->bytes = requestBytes(req->shot, r->denoise());
  int albedo, normal;
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
  else if (r->denoise() && (S->denoisers.empty() || req->shot.frames < 2 || !guideImages(req->shot, &albedo, &normal)))
    reason = ASUNA_ERR_INVALID;  // no denoiser, fewer than two frames or no albedo / normal channel
  else if (r->bytes + (S->scenes[req->scene].dev ? 0 : S->scenes[req->scene].estimate) > S->opts.memory_budget)
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
  std::lock_guard<std::mutex> io(r->io);
  if (r->status != ASUNA_OK || !r->film[0])
    return asuna::fail(ASUNA_ERR_INVALID, "request %llu has no film", (unsigned long long)id);
  if (r->finish < 0) return asuna::fail(ASUNA_ERR_INVALID, "request %llu is not finished", (unsigned long long)id);
  if (!host_rgba) return asuna::fail(ASUNA_ERR_INVALID, "null output");
  if (image < 0 || image >= ASUNA_NUM_OUTPUT_IMAGES) return asuna::fail(ASUNA_ERR_INVALID, "image %d out of range", image);
  // the worker synchronised its stream before marking the request finished
  float* src = nullptr;
  if (image == 0 && r->denoised) {
    src = r->denoised;
  } else {
    int rc = asuna_film_image(r->film[0], image, &src);
    if (rc) return rc;
  }
  ASUNA_CUDA_TRY(cudaSetDevice(S->opts.device));
  ASUNA_CUDA_TRY(cudaMemcpyAsync(host_rgba, src, size_t(r->shot.width) * r->shot.height * 16,
                                 cudaMemcpyDeviceToHost, S->readStream));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(S->readStream));
  return ASUNA_OK;
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
    if (r->charged) S->memUsed -= r->bytes;
    r->charged = false;
  }
  {
    std::lock_guard<std::mutex> io(r->io);  // after any read in progress
    freeRequest(*r);
  }
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
  std::memset(out, 0, sizeof(*out));
  out->admitted = S->admitted;
  out->rejected = S->rejected;
  out->pending = S->pending.size();
  out->samples = S->samples;
  out->memory_used = S->memUsed;
  out->elapsed_s = S->now();
  out->scenes_built = S->built;
  out->scenes_evicted = S->evicted;
  out->denoised = S->denoised;
  for (const SceneEntry& e : S->scenes)
    if (e.dev) out->scene_bytes += e.bytes;
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
  for (auto& kv : S->byId) freeRequest(*kv.second);
  for (auto* d : S->denoisers) asuna_denoiser_destroy(d);
  for (auto& e : S->scenes)
    if (e.dev) asuna_scene_destroy(e.dev);
  for (auto* c : S->ctxs) asuna_ctx_destroy(c);
  if (S->readStream) cudaStreamDestroy(S->readStream);
  delete S;
  return ASUNA_OK;
}

}  // extern "C"
