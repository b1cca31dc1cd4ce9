// ibl_server.cu -- continuous probe re-baking under a device-memory budget.
//
// Requests arrive at any time (althea_ibl_server_submit).  A request is
// admitted as soon as a slot (a CUDA stream) is free and its device block
// (env chain + outputs + irradiance scratch) fits the budget; otherwise it
// waits in FIFO order and is admitted by a later submit or poll once earlier
// requests retire.  Admitted requests run concurrently, one stream each:
//   H2D env -> chain build -> prefilter (all mips) -> irradiance -> D2H
// and a host callback on the stream stamps the completion time.  Device
// blocks come from a pool with exact-size free lists: memory is allocated once
// per size class and reused, so the request path issues no cudaFree (which
// would synchronise the device); free blocks of other sizes are released only
// when a new size class would otherwise exceed the budget.
//
// Resident maps: althea_ibl_server_register_env uploads an env map once and
// keeps it on the device (its bytes count against the budget); a request that
// names it copies it on the device into its own chain, adds the request's sun
// lobes (ibl_suns.cu) and bakes, so no env map crosses the host link.
//
// Host code only; the kernels are the single-probe ones (ibl_plain.cu, or
// ibl_tc.cu when the server runs the precision path), whose results do not
// depend on what else runs on the device.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <deque>
#include <map>
#include <new>
#include <vector>

#include "althea_ibl.h"
#include "ibl_internal.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct Layout {
  size_t chain_off, mips_off, irr_off, ws_off, total;
  size_t mips_bytes, irr_bytes, ws_bytes;
  int mip_w[ALTHEA_IBL_MAX_MIPS], mip_h[ALTHEA_IBL_MAX_MIPS];
};

// Mip targets of a request (mips from W/2 x H/2, roughness m/(M-1)) inside a block.
void mip_targets(const Layout& L, char* base, int mips, althea_ibl_mip_target* out) {
  size_t off = L.mips_off;
  for (int m = 0; m < mips; ++m) {
    out[m].out_dev = base ? reinterpret_cast<float*>(base + off) : nullptr;
    out[m].pitch_bytes = (size_t)L.mip_w[m] * 16;
    out[m].width = L.mip_w[m];
    out[m].height = L.mip_h[m];
    out[m].roughness = mips > 1 ? (float)m / (float)(mips - 1) : 0.0f;
    off += (size_t)L.mip_w[m] * L.mip_h[m] * 16;
  }
}

struct Slot {
  cudaStream_t stream = nullptr;
  bool busy = false;
  std::atomic<int> done{0};
  double done_s = 0.0;
  althea_ibl_completion info{};
  void* block = nullptr;
  size_t bytes = 0;
  int status = ALTHEA_IBL_OK;
  int env_width = 0, env_height = 0, mip_count = 0;  // shape of the request in flight
  int env_id = 0;                                    // resident map it reads, or 0
};

struct ResidentEnv {
  float* level0 = nullptr;  // RGBA32F, tightly packed
  int width = 0, height = 0;
  size_t bytes = 0;
  int users = 0;            // queued and running requests that read it
};

struct Pending {
  althea_ibl_request req;
  double submit_s;
};

}  // namespace

struct althea_ibl_server {
  althea_ibl_server_config cfg{};
  std::vector<Slot*> slots;
  std::deque<Pending> queue;
  std::deque<althea_ibl_completion> finished;  // retired, not yet returned
  std::map<size_t, std::vector<void*>> free_blocks;
  size_t reserved = 0, in_use = 0, peak = 0;
  uint64_t completed = 0, rejected = 0;
  std::map<int, ResidentEnv> resident;
  size_t resident_bytes = 0;
  int next_env_id = 1;
};

namespace {

void CUDART_CB on_done(void* p) {
  Slot* s = static_cast<Slot*>(p);
  s->done_s = now_s();
  s->done.store(1, std::memory_order_release);
}

Layout layout_for(const althea_ibl_server* s, int w, int h, int mips) {
  Layout L{};
  size_t off = 0;
  L.chain_off = off;
  off = align256(off + althea_ibl_chain_texels(w, h) * 16);
  L.mips_off = off;
  size_t mb = 0;
  int fw = w >> 1 < 1 ? 1 : w >> 1, fh = h >> 1 < 1 ? 1 : h >> 1;
  for (int m = 0; m < mips; ++m) {
    L.mip_w[m] = (fw >> m) < 1 ? 1 : (fw >> m);
    L.mip_h[m] = (fh >> m) < 1 ? 1 : (fh >> m);
    mb += (size_t)L.mip_w[m] * L.mip_h[m] * 16;
  }
  L.mips_bytes = mb;
  off = align256(off + mb);
  L.irr_off = off;
  L.irr_bytes = (size_t)s->cfg.irradiance_width * s->cfg.irradiance_height * 16;
  off = align256(off + L.irr_bytes);
  L.ws_off = off;
  if (s->cfg.path == ALTHEA_IBL_PATH_PRECISION) {
    althea_ibl_mip_target mt[ALTHEA_IBL_MAX_MIPS];
    mip_targets(L, nullptr, mips, mt);
    L.ws_bytes = ibl::tc_workspace_bytes(w, h, mt, mips, nullptr, s->cfg.irradiance_width,
                                         s->cfg.irradiance_height, -1);
    if (L.ws_bytes == 0) {  // unsupported shape: can never be admitted
      L.total = (size_t)-1;
      return L;
    }
  } else {
    L.ws_bytes =
        ibl::irr_plan(w, h, s->cfg.irradiance_width, s->cfg.irradiance_height).workspace;
  }
  off = align256(off + L.ws_bytes);
  L.total = off;
  return L;
}

// Block of exactly `bytes` from the pool; false when it cannot fit now.
// Frees idle pool blocks until `extra` more bytes fit the budget beside the
// reserved blocks and the resident maps; false when they cannot.
bool make_room(althea_ibl_server* s, size_t extra) {
  while (s->reserved + s->resident_bytes + extra > s->cfg.budget_bytes) {
    bool freed = false;
    for (auto& kv : s->free_blocks) {
      if (!kv.second.empty()) {
        cudaFree(kv.second.back());
        kv.second.pop_back();
        s->reserved -= kv.first;
        freed = true;
        break;
      }
    }
    if (!freed) return false;
  }
  return true;
}

bool pool_acquire(althea_ibl_server* s, size_t bytes, void** out) {
  if (s->in_use + s->resident_bytes + bytes > s->cfg.budget_bytes) return false;
  auto it = s->free_blocks.find(bytes);
  if (it != s->free_blocks.end() && !it->second.empty()) {
    *out = it->second.back();
    it->second.pop_back();
    s->in_use += bytes;
    if (s->in_use > s->peak) s->peak = s->in_use;
    return true;
  }
  // A new block: release idle blocks of other sizes until it fits.
  if (!make_room(s, bytes)) return false;
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  s->reserved += bytes;
  s->in_use += bytes;
  if (s->in_use > s->peak) s->peak = s->in_use;
  *out = p;
  return true;
}

void pool_release(althea_ibl_server* s, void* p, size_t bytes) {
  s->free_blocks[bytes].push_back(p);
  s->in_use -= bytes;
}

int start(althea_ibl_server* s, Slot* slot, const Pending& pend, const Layout& L) {
  ibl::NvtxRange nvtx_range("server request");
  const althea_ibl_request& r = pend.req;
  cudaStream_t st = slot->stream;
  char* base = static_cast<char*>(slot->block);
  float* chain = reinterpret_cast<float*>(base + L.chain_off);
  int status = ALTHEA_IBL_OK;
  cudaError_t e = cudaSuccess;
  if (r.env_id) {
    // the resident map plus this request's suns, written into the request's chain
    const ResidentEnv& env = s->resident.at(r.env_id);
    status = ibl::launch_apply_suns(env.level0, chain, r.env_width, r.env_height, r.suns,
                                    r.sun_count, st);
  } else {
    e = cudaMemcpyAsync(chain, r.env_host, (size_t)r.env_width * r.env_height * 16,
                        cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) status = ibl::cuda_status(e, "server env upload");
    if (!status && r.sun_count > 0)
      status = ibl::launch_apply_suns(chain, chain, r.env_width, r.env_height, r.suns,
                                      r.sun_count, st);
  }
  if (!status) status = ibl::launch_build_chain(chain, r.env_width, r.env_height, chain, st);
  althea_ibl_mip_target mips[ALTHEA_IBL_MAX_MIPS];
  mip_targets(L, base, r.mip_count, mips);
  if (s->cfg.path == ALTHEA_IBL_PATH_PRECISION) {
    if (!status)
      status = ibl::tc_bake(chain, r.env_width, r.env_height, mips, r.mip_count, nullptr,
                            r.irradiance_host ? reinterpret_cast<float*>(base + L.irr_off)
                                              : nullptr,
                            s->cfg.irradiance_width, s->cfg.irradiance_height,
                            (size_t)s->cfg.irradiance_width * 16, -1, base + L.ws_off,
                            L.ws_bytes, ALTHEA_IBL_FORMAT_RGBA32F, st);
  } else {
    if (!status)
      status = ibl::launch_prefilter(chain, r.env_width, r.env_height, mips, r.mip_count,
                                     s->cfg.samples, s->cfg.generator, st);
    if (!status && r.irradiance_host)
      status = ibl::launch_irradiance(chain, r.env_width, r.env_height,
                                      reinterpret_cast<float*>(base + L.irr_off),
                                      s->cfg.irradiance_width, s->cfg.irradiance_height,
                                      (size_t)s->cfg.irradiance_width * 16, base + L.ws_off, st);
  }
  if (!status && r.mips_host && L.mips_bytes) {
    e = cudaMemcpyAsync(r.mips_host, base + L.mips_off, L.mips_bytes, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) status = ibl::cuda_status(e, "server mips download");
  }
  if (!status && r.irradiance_host) {
    e = cudaMemcpyAsync(r.irradiance_host, base + L.irr_off, L.irr_bytes, cudaMemcpyDeviceToHost,
                        st);
    if (e != cudaSuccess) status = ibl::cuda_status(e, "server irradiance download");
  }
  slot->status = status;
  slot->done.store(0, std::memory_order_relaxed);
  e = cudaLaunchHostFunc(st, on_done, slot);
  if (e != cudaSuccess) {
    // No callback queued: wait here so the slot can still be retired.
    cudaStreamSynchronize(st);
    on_done(slot);
    if (!slot->status) slot->status = ibl::cuda_status(e, "server completion callback");
  }
  return status;
}

void admit(althea_ibl_server* s) {
  while (!s->queue.empty()) {
    const Pending& head = s->queue.front();
    Layout L = layout_for(s, head.req.env_width, head.req.env_height, head.req.mip_count);
    if (L.total + s->resident_bytes > s->cfg.budget_bytes) {  // cannot fit beside the maps
      althea_ibl_completion c{};
      c.tag = head.req.tag;
      c.status = ALTHEA_IBL_ERR_BUDGET;
      c.submit_s = c.start_s = c.done_s = head.submit_s;
      s->finished.push_back(c);
      s->rejected++;
      if (head.req.env_id) s->resident[head.req.env_id].users--;
      s->queue.pop_front();
      continue;
    }
    Slot* free_slot = nullptr;
    for (Slot* sl : s->slots)
      if (!sl->busy) {
        free_slot = sl;
        break;
      }
    if (!free_slot) return;
    void* block = nullptr;
    if (!pool_acquire(s, L.total, &block)) return;  // FIFO: wait for memory
    free_slot->busy = true;
    free_slot->block = block;
    free_slot->bytes = L.total;
    free_slot->info.tag = head.req.tag;
    free_slot->info.submit_s = head.submit_s;
    free_slot->info.start_s = now_s();
    free_slot->env_width = head.req.env_width;
    free_slot->env_height = head.req.env_height;
    free_slot->mip_count = head.req.mip_count;
    free_slot->env_id = head.req.env_id;
    start(s, free_slot, head, L);
    s->queue.pop_front();
  }
}

void retire(althea_ibl_server* s) {
  for (Slot* sl : s->slots) {
    if (!sl->busy || !sl->done.load(std::memory_order_acquire)) continue;
    althea_ibl_completion c = sl->info;
    c.done_s = sl->done_s;
    c.status = sl->status;
    if (s->cfg.path == ALTHEA_IBL_PATH_PRECISION && c.status == ALTHEA_IBL_OK) {
      // the precision kernels' bounded waits report through the workspace's
      // first word; the slot's stream has finished, so this read is immediate
      int flag = 0;
      Layout L = layout_for(s, sl->env_width, sl->env_height, sl->mip_count);
      if (cudaMemcpyAsync(&flag, static_cast<char*>(sl->block) + L.ws_off, sizeof(int),
                          cudaMemcpyDeviceToHost, sl->stream) != cudaSuccess ||
          cudaStreamSynchronize(sl->stream) != cudaSuccess || flag)
        c.status = ALTHEA_IBL_ERR_CUDA;
    }
    s->finished.push_back(c);
    pool_release(s, sl->block, sl->bytes);
    if (sl->env_id) s->resident[sl->env_id].users--;
    sl->env_id = 0;
    sl->block = nullptr;
    sl->busy = false;
    s->completed++;
  }
}

int check_request(const althea_ibl_server* s, const althea_ibl_request* r) {
  if (!r) return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null request");
  if (r->env_id) {
    auto it = s->resident.find(r->env_id);
    if (it == s->resident.end())
      return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "env_id %d is not registered",
                            r->env_id);
    if (it->second.width != r->env_width || it->second.height != r->env_height)
      return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT,
                            "request size %dx%d; resident map %d is %dx%d", r->env_width,
                            r->env_height, r->env_id, it->second.width, it->second.height);
  } else if (!r->env_host) {
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "request: no env_host and no env_id");
  }
  if (r->sun_count < 0 || r->sun_count > ALTHEA_IBL_MAX_SUNS)
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "request sun_count %d outside 0..%d",
                          r->sun_count, ALTHEA_IBL_MAX_SUNS);
  int st = ibl::check_env(r->env_width, r->env_height);
  if (st) return st;
  if (r->mip_count < 1 || r->mip_count > ALTHEA_IBL_MAX_MIPS)
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "request mip_count %d", r->mip_count);
  if (r->irradiance_host)
    return ibl::check_irradiance_args(r->env_width, r->env_height, s->cfg.irradiance_width,
                                      s->cfg.irradiance_height);
  return ALTHEA_IBL_OK;
}

}  // namespace

extern "C" double althea_ibl_server_now(void) { return now_s(); }

extern "C" int althea_ibl_server_create(const althea_ibl_server_config* cfg,
                                        althea_ibl_server** out) {
  if (!cfg || !out) return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (cfg->max_inflight < 1 || cfg->max_inflight > 256 || cfg->budget_bytes == 0 ||
      cfg->samples < 1 || cfg->samples > (1 << 24) ||
      (cfg->generator != ALTHEA_IBL_GEN_REF_HASH && cfg->generator != ALTHEA_IBL_GEN_HAMMERSLEY) ||
      cfg->irradiance_width < 1 || cfg->irradiance_height < 1 ||
      (cfg->path != ALTHEA_IBL_PATH_PLAIN && cfg->path != ALTHEA_IBL_PATH_PRECISION))
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "server config");
  althea_ibl_server* s = new (std::nothrow) althea_ibl_server();
  if (!s) return ibl::set_error(ALTHEA_IBL_ERR_OUT_OF_MEMORY, "host allocation");
  s->cfg = *cfg;
  for (int i = 0; i < cfg->max_inflight; ++i) {
    Slot* sl = new (std::nothrow) Slot();
    if (!sl || cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete sl;
      althea_ibl_server_destroy(s);
      return ibl::set_error(ALTHEA_IBL_ERR_CUDA, "server stream creation");
    }
    s->slots.push_back(sl);
  }
  *out = s;
  return ALTHEA_IBL_OK;
}

extern "C" size_t althea_ibl_server_request_bytes(const althea_ibl_server* s, int w, int h,
                                                  int mips) {
  if (!s || ibl::check_env(w, h) || mips < 1 || mips > ALTHEA_IBL_MAX_MIPS) return 0;
  const size_t total = layout_for(s, w, h, mips).total;
  return total == (size_t)-1 ? 0 : total;
}

extern "C" int althea_ibl_server_submit(althea_ibl_server* s, const althea_ibl_request* r) {
  if (!s) return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null server");
  int st = check_request(s, r);
  if (st) return st;
  const size_t total = layout_for(s, r->env_width, r->env_height, r->mip_count).total;
  if (total == (size_t)-1) {
    // the precision planner refused the shape; the last error holds its reason
    s->rejected++;
    return ALTHEA_IBL_ERR_UNSUPPORTED;
  }
  if (total + s->resident_bytes > s->cfg.budget_bytes) {
    s->rejected++;
    return ibl::set_error(ALTHEA_IBL_ERR_BUDGET, "request needs more device memory than the "
                                                 "server budget of %zu bytes leaves beside "
                                                 "%zu bytes of resident maps",
                          s->cfg.budget_bytes, s->resident_bytes);
  }
  if (r->env_id) s->resident[r->env_id].users++;
  s->queue.push_back(Pending{*r, now_s()});
  retire(s);
  admit(s);
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_server_poll(althea_ibl_server* s, althea_ibl_completion* out, int max,
                                      int* n) {
  if (!s || !n || (max > 0 && !out))
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null argument");
  retire(s);
  admit(s);
  int k = 0;
  while (k < max && !s->finished.empty()) {
    out[k++] = s->finished.front();
    s->finished.pop_front();
  }
  *n = k;
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_server_get_stats(const althea_ibl_server* s, althea_ibl_server_stats* st) {
  if (!s || !st) return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null argument");
  int inflight = 0;
  for (Slot* sl : s->slots) inflight += sl->busy ? 1 : 0;
  st->inflight = inflight;
  st->queued = (int)s->queue.size();
  st->bytes_in_use = s->in_use;
  st->bytes_reserved = s->reserved;
  st->peak_bytes_in_use = s->peak;
  st->completed = s->completed;
  st->rejected = s->rejected;
  st->bytes_resident = s->resident_bytes;
  st->resident_maps = (int)s->resident.size();
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_server_register_env(althea_ibl_server* s, const float* rgba, int w,
                                              int h, int src_is_device, int* env_id_out) {
  if (!s || !rgba || !env_id_out)
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null argument");
  *env_id_out = 0;
  int st = ibl::check_env(w, h);
  if (st) return st;
  const size_t bytes = (size_t)w * h * 16;
  if (!make_room(s, bytes))
    return ibl::set_error(ALTHEA_IBL_ERR_BUDGET,
                          "a %dx%d map (%zu bytes) does not fit the budget of %zu bytes beside "
                          "%zu bytes in use and %zu resident",
                          w, h, bytes, s->cfg.budget_bytes, s->in_use, s->resident_bytes);
  ResidentEnv env;
  env.width = w;
  env.height = h;
  env.bytes = bytes;
  cudaError_t e = cudaMalloc(&env.level0, bytes);
  if (e != cudaSuccess) return ibl::cuda_status(e, "resident map allocation");
  e = cudaMemcpy(env.level0, rgba, bytes,
                 src_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(env.level0);
    return ibl::cuda_status(e, "resident map upload");
  }
  const int id = s->next_env_id++;
  s->resident[id] = env;
  s->resident_bytes += bytes;
  *env_id_out = id;
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_server_unregister_env(althea_ibl_server* s, int env_id) {
  if (!s) return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null server");
  retire(s);  // requests that finished no longer hold the map
  auto it = s->resident.find(env_id);
  if (it == s->resident.end())
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "env_id %d is not registered",
                          env_id);
  if (it->second.users > 0)
    return ibl::set_error(ALTHEA_IBL_ERR_NOT_READY, "resident map %d is used by %d requests",
                          env_id, it->second.users);
  cudaFree(it->second.level0);
  s->resident_bytes -= it->second.bytes;
  s->resident.erase(it);
  admit(s);  // memory freed: queued requests may fit now
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_server_destroy(althea_ibl_server* s) {
  if (!s) return ALTHEA_IBL_OK;
  for (Slot* sl : s->slots) {
    if (sl->stream) cudaStreamSynchronize(sl->stream);
  }
  retire(s);
  for (Slot* sl : s->slots) {
    if (sl->block) cudaFree(sl->block);
    if (sl->stream) cudaStreamDestroy(sl->stream);
    delete sl;
  }
  for (auto& kv : s->free_blocks)
    for (void* p : kv.second) cudaFree(p);
  for (auto& kv : s->resident) cudaFree(kv.second.level0);
  delete s;
  return ALTHEA_IBL_OK;
}
