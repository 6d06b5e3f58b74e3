// Request server over resident worlds: continuous batching of render and edit requests.
//
// The reference renders one frame per glDrawArrays and edits the world on the CPU between
// frames (main.cpp:58-73, controls.cpp:100-110).  Here requests arrive at any time
// (vrt_server_submit, thread-safe) and vrt_server_poll:
//   - retires finished launches (event query, never blocks) and frees their images;
//   - admits queued requests into free slots (a slot = a stream + a renderer) while the
//     memory budget (resident worlds + images in flight) allows;
//   - batches the renders of one world into one launch (vrt_render_batch), so requests
//     that arrive while others run join the next free slot and overlap them on the device;
//     a partial batch may wait max_wait_us for company, and max_batch_pixels caps a launch's
//     work so that a request arriving under load waits behind less of it;
//   - keeps the order of each world's requests: an edit waits (on the device, through
//     events) for every earlier render of its world, and later renders wait for it.
// Requests larger than the whole budget complete with VRT_EBUDGET.
// Images render straight into page-locked host memory by default (the kernels store the
// pixels over the host link): the request's own buffer when it is page-locked, else the
// slot's.  image_memory = 1 renders into device memory and copies to the slot's buffer.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "vrt_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Queued {
    vrt_request req;
    double submit_ms;
    uint64_t bytes;  // image bytes (render)
};

struct WorldEntry {
    vrt_world* w = nullptr;
    cudaEvent_t edit_event = nullptr;  // last edit of this world
    bool has_edit = false;
};

struct Slot {
    cudaStream_t stream = nullptr;
    vrt_renderer* renderer = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    int world_id = -1;
    bool is_edit = false;
    std::vector<Queued> reqs;
    std::vector<uint8_t*> d_images;   // device images (image_memory = 1), else NULL
    std::vector<uint64_t> image_bytes;
    std::vector<char> in_place;       // rendered straight into the request's own buffer
    uint64_t* d_stats = nullptr;  // per request VRT_STAT_COUNT counters
    uint64_t* h_stats = nullptr;  // pinned
    int stats_cap = 0;
    uint8_t* h_staging = nullptr;  // pinned
    uint8_t* staging_dev = nullptr;  // h_staging's address in the device's address space
    uint64_t staging_cap = 0;
    double start_ms = 0;
    uint64_t bytes_in_flight = 0;
};

// A size-bucketed cache of device image buffers (no cudaMalloc on the steady path).
struct ImagePool {
    std::vector<std::pair<uint64_t, uint8_t*>> free_list;
    uint8_t* get(uint64_t bytes) {
        for (size_t i = 0; i < free_list.size(); i++)
            if (free_list[i].first == bytes) {
                uint8_t* p = free_list[i].second;
                free_list.erase(free_list.begin() + i);
                return p;
            }
        uint8_t* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return p;
    }
    void put(uint64_t bytes, uint8_t* p) { free_list.emplace_back(bytes, p); }
    ~ImagePool() {
        for (auto& f : free_list) cudaFree(f.second);
    }
};

}  // namespace

struct vrt_server {
    vrt_server_config cfg;
    Clock::time_point t0;
    std::mutex mu;  // guards queue, done and the worlds list (not the entries it points to)
    std::deque<Queued> queue;
    // Entries are allocated one by one and never move: vrt_server_add_world may grow the
    // list from any thread while the polling thread works on an entry it looked up.
    std::vector<std::unique_ptr<WorldEntry>> worlds;
    std::vector<Slot> slots;
    ImagePool pool;
    uint64_t world_bytes = 0;
    uint64_t image_bytes = 0;  // images in flight
    std::vector<vrt_completion> done;
    double now() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
};

using namespace vrt;

// The entry of world `wid`: looked up under the lock, used without it (the entry's world
// and event never change after vrt_server_add_world; has_edit is the polling thread's).
static WorldEntry* world_entry(vrt_server* s, int wid) {
    std::lock_guard<std::mutex> lk(s->mu);
    return s->worlds[wid].get();
}

static void retire(vrt_server* s, Slot& sl) {
    double t = s->now();
    for (size_t i = 0; i < sl.reqs.size(); i++) {
        const Queued& q = sl.reqs[i];
        vrt_completion c{};
        c.user_tag = q.req.user_tag;
        c.status = VRT_OK;
        c.kind = q.req.kind;
        c.submit_ms = q.submit_ms;
        c.start_ms = sl.start_ms;
        c.done_ms = t;
        if (q.req.kind == VRT_REQ_RENDER) {
            c.rays = sl.h_stats[i * VRT_STAT_COUNT + VRT_STAT_RAYS];
            if (q.req.host_rgba && !sl.in_place[i]) {
                uint64_t off = 0;
                for (size_t j = 0; j < i; j++) off += sl.image_bytes[j];
                std::memcpy(q.req.host_rgba, sl.h_staging + off, sl.image_bytes[i]);
            }
            if (sl.d_images[i]) s->pool.put(sl.image_bytes[i], sl.d_images[i]);
        }
        s->done.push_back(c);
    }
    s->image_bytes -= sl.bytes_in_flight;
    sl.bytes_in_flight = 0;
    sl.reqs.clear();
    sl.d_images.clear();
    sl.image_bytes.clear();
    sl.in_place.clear();
    sl.busy = false;
}

// Make stream `st` wait for every in-flight render of world `wid` (except on slot `self`).
static int wait_for_renders(vrt_server* s, int wid, cudaStream_t st, int self) {
    for (size_t i = 0; i < s->slots.size(); i++) {
        Slot& o = s->slots[i];
        if ((int)i == self || !o.busy || o.world_id != wid) continue;
        VRT_CUDA(cudaStreamWaitEvent(st, o.done, 0));
    }
    return VRT_OK;
}

static int launch_edit(vrt_server* s, int si, const Queued& q) {
    Slot& sl = s->slots[si];
    WorldEntry& we = *world_entry(s, q.req.world_id);
    int st = wait_for_renders(s, q.req.world_id, sl.stream, si);
    if (st) return st;
    if (we.has_edit) VRT_CUDA(cudaStreamWaitEvent(sl.stream, we.edit_event, 0));
    st = vrt_remove_sphere(we.w, q.req.cx, q.req.cy, q.req.cz, q.req.radius, we.w->has_depth_field, sl.stream);
    if (st) return st;
    VRT_CUDA(cudaEventRecord(we.edit_event, sl.stream));
    we.has_edit = true;
    VRT_CUDA(cudaEventRecord(sl.done, sl.stream));
    sl.busy = true;
    sl.is_edit = true;
    sl.world_id = q.req.world_id;
    sl.reqs.assign(1, q);
    sl.start_ms = s->now();
    return VRT_OK;
}

static int ensure_slot_buffers(Slot& sl, int n, uint64_t bytes) {
    if (n > sl.stats_cap) {
        cudaFree(sl.d_stats);
        cudaFreeHost(sl.h_stats);
        sl.d_stats = nullptr;
        sl.h_stats = nullptr;
        sl.stats_cap = 0;
        VRT_CUDA(cudaMalloc(&sl.d_stats, sizeof(uint64_t) * VRT_STAT_COUNT * n));
        VRT_CUDA(cudaMallocHost(&sl.h_stats, sizeof(uint64_t) * VRT_STAT_COUNT * n));
        sl.stats_cap = n;
    }
    if (bytes > sl.staging_cap) {
        cudaFreeHost(sl.h_staging);
        sl.h_staging = nullptr;
        sl.staging_cap = 0;
        VRT_CUDA(cudaMallocHost(&sl.h_staging, bytes));
        void* dev = nullptr;
        VRT_CUDA(cudaHostGetDevicePointer(&dev, sl.h_staging, 0));
        sl.staging_dev = static_cast<uint8_t*>(dev);
        sl.staging_cap = bytes;
    }
    return VRT_OK;
}

// The address the kernel can store a request's image to when the request's own buffer is
// page-locked host memory (mapped into the device's address space), else NULL.
static uint8_t* mapped_host_image(uint8_t* host) {
    if (!host) return nullptr;
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, host) != cudaSuccess) {
        (void)cudaGetLastError();  // pageable memory
        return nullptr;
    }
    if (pa.type != cudaMemoryTypeHost || !pa.devicePointer || ((uintptr_t)pa.devicePointer & 3)) return nullptr;
    return static_cast<uint8_t*>(pa.devicePointer);
}

static void release_images(vrt_server* s, Slot& sl) {
    for (size_t i = 0; i < sl.d_images.size(); i++)
        if (sl.d_images[i]) s->pool.put(sl.image_bytes[i], sl.d_images[i]);
    sl.d_images.clear();
    sl.image_bytes.clear();
    sl.in_place.clear();
}

static int launch_renders(vrt_server* s, int si, std::vector<Queued>& batch) {
    Slot& sl = s->slots[si];
    const int wid = batch[0].req.world_id;
    WorldEntry& we = *world_entry(s, wid);
    const bool on_device = s->cfg.image_memory == 1;
    uint64_t total = 0;
    for (auto& q : batch) total += q.bytes;
    int st = ensure_slot_buffers(sl, (int)batch.size(), total);
    if (st) return st;
    std::vector<vrt_view> views(batch.size());
    release_images(s, sl);
    uint64_t off = 0;
    for (size_t i = 0; i < batch.size(); i++) {
        uint8_t* img = nullptr;
        uint8_t* dst = nullptr;
        bool in_place = false;
        if (on_device) {
            img = s->pool.get(batch[i].bytes);
            if (!img) {
                release_images(s, sl);
                return set_error(VRT_ENOMEM, "image allocation failed");
            }
            dst = img;
        } else {
            dst = mapped_host_image(batch[i].req.host_rgba);
            in_place = dst != nullptr;
            if (!dst) dst = sl.staging_dev + off;  // image bytes are multiples of 4: aligned
        }
        off += batch[i].bytes;
        sl.d_images.push_back(img);
        sl.image_bytes.push_back(batch[i].bytes);
        sl.in_place.push_back(in_place);
        vrt_view& v = views[i];
        std::memset(&v, 0, sizeof(v));
        v.world = we.w;
        v.uniforms = batch[i].req.uniforms;
        v.width = batch[i].req.width;
        v.height = batch[i].req.height;
        v.d_rgba = dst;
        v.d_stats = sl.d_stats + i * VRT_STAT_COUNT;
    }
    if (we.has_edit) VRT_CUDA(cudaStreamWaitEvent(sl.stream, we.edit_event, 0));
    VRT_CUDA(cudaMemsetAsync(sl.d_stats, 0, sizeof(uint64_t) * VRT_STAT_COUNT * batch.size(), sl.stream));
    st = vrt_render_batch(sl.renderer, views.data(), (int)views.size(), nullptr, sl.stream);
    if (st) {
        release_images(s, sl);
        return st;
    }
    if (on_device) {
        off = 0;
        for (size_t i = 0; i < batch.size(); i++) {
            VRT_CUDA(cudaMemcpyAsync(sl.h_staging + off, sl.d_images[i], sl.image_bytes[i], cudaMemcpyDeviceToHost,
                                     sl.stream));
            off += sl.image_bytes[i];
        }
    }
    VRT_CUDA(cudaMemcpyAsync(sl.h_stats, sl.d_stats, sizeof(uint64_t) * VRT_STAT_COUNT * batch.size(),
                             cudaMemcpyDeviceToHost, sl.stream));
    VRT_CUDA(cudaEventRecord(sl.done, sl.stream));
    sl.busy = true;
    sl.is_edit = false;
    sl.world_id = wid;
    sl.reqs = batch;
    sl.start_ms = s->now();
    sl.bytes_in_flight = total;
    s->image_bytes += total;
    return VRT_OK;
}

static inline uint64_t pixels_of(const vrt_request& r) { return (uint64_t)r.width * (uint64_t)r.height; }

// Would a batch of n requests and px pixels exceed max_batch_pixels by taking r?  The first
// request of a batch always fits.
static inline bool over_pixel_cap(const vrt_server* s, int n, uint64_t px, const vrt_request& r) {
    return s->cfg.max_batch_pixels > 0 && n > 0 && px + pixels_of(r) > (uint64_t)s->cfg.max_batch_pixels;
}

// Take the next launch off the queue for a free slot; returns false when nothing can start.
static bool admit(vrt_server* s, int si, int* status) {
    std::vector<Queued> batch;
    Queued edit;
    bool is_edit = false;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->queue.empty()) return false;
        // a world's requests keep their order: skip worlds that have an earlier request
        // still waiting behind the budget, and never move a render past an edit
        std::vector<char> blocked(s->worlds.size(), 0);
        for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
            const int wid = it->req.world_id;
            if (blocked[wid]) continue;
            if (it->req.kind == VRT_REQ_EDIT) {
                edit = *it;
                s->queue.erase(it);
                is_edit = true;
                break;
            }
            uint64_t cap = s->cfg.memory_budget_bytes - s->world_bytes;
            if (s->image_bytes + it->bytes > cap) {
                blocked[wid] = 1;
                continue;
            }
            if (s->cfg.max_wait_us > 0 && s->now() - it->submit_ms < 1e-3 * s->cfg.max_wait_us) {
                // a young partial batch waits for company (a full one, or one that meets the
                // world's next edit, goes now)
                int n = 0;
                uint64_t px = 0;
                bool closed = false;
                for (auto jt = it; jt != s->queue.end() && n < s->cfg.max_batch; ++jt) {
                    if (jt->req.world_id != wid) continue;
                    if (jt->req.kind == VRT_REQ_EDIT || over_pixel_cap(s, n, px, jt->req)) {
                        closed = true;  // the batch cannot grow any further
                        break;
                    }
                    px += pixels_of(jt->req);
                    n++;
                }
                if (n < s->cfg.max_batch && !closed) {
                    blocked[wid] = 1;
                    continue;
                }
            }
            // gather this world's renders in order, up to the first edit of the world
            uint64_t used = s->image_bytes, px = 0;
            for (auto jt = it; jt != s->queue.end() && (int)batch.size() < s->cfg.max_batch;) {
                if (jt->req.world_id != wid) { ++jt; continue; }
                if (jt->req.kind == VRT_REQ_EDIT) break;
                if (used + jt->bytes > cap) break;
                if (over_pixel_cap(s, (int)batch.size(), px, jt->req)) break;
                used += jt->bytes;
                px += pixels_of(jt->req);
                batch.push_back(*jt);
                jt = s->queue.erase(jt);
            }
            break;
        }
    }
    if (is_edit) {
        *status = launch_edit(s, si, edit);
        return *status == VRT_OK;
    }
    if (batch.empty()) return false;
    *status = launch_renders(s, si, batch);
    if (*status) {
        // put the requests back at the front, in order
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto it = batch.rbegin(); it != batch.rend(); ++it) s->queue.push_front(*it);
        return false;
    }
    return true;
}

extern "C" {

int vrt_server_create(const vrt_server_config* cfg, vrt_server** out) {
    if (!cfg || !out) return set_error(VRT_EINVAL, "NULL argument");
    *out = nullptr;
    if (cfg->slots < 1 || cfg->slots > 64 || cfg->max_batch < 1 || cfg->memory_budget_bytes == 0 ||
        cfg->max_wait_us < 0 || (cfg->image_memory != 0 && cfg->image_memory != 1) || cfg->max_batch_pixels < 0)
        return set_error(VRT_EINVAL, "bad server config (slots 1-64, max_batch >= 1, budget > 0, max_wait_us >= 0, "
                                     "max_batch_pixels >= 0, "
                                     "image_memory 0 or 1)");
    vrt_server* s = new vrt_server();
    s->cfg = *cfg;
    s->t0 = Clock::now();
    s->slots.resize(cfg->slots);
    for (auto& sl : s->slots) {
        cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        int st = e == cudaSuccess ? vrt_renderer_create(&sl.renderer) : cuda_error(e, "slot");
        if (st) {
            vrt_server_destroy(s);
            return st;
        }
    }
    *out = s;
    return VRT_OK;
}

int vrt_server_destroy(vrt_server* s) {
    if (!s) return VRT_OK;
    for (auto& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        release_images(s, sl);
        vrt_renderer_destroy(sl.renderer);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        cudaFree(sl.d_stats);
        cudaFreeHost(sl.h_stats);
        cudaFreeHost(sl.h_staging);
    }
    for (auto& we : s->worlds)
        if (we->edit_event) cudaEventDestroy(we->edit_event);
    delete s;
    return VRT_OK;
}

int vrt_server_add_world(vrt_server* s, vrt_world* w, int32_t* id) {
    if (!s || !w || !id) return set_error(VRT_EINVAL, "NULL argument");
    std::unique_ptr<WorldEntry> we(new WorldEntry());
    we->w = w;
    VRT_CUDA(cudaEventCreateWithFlags(&we->edit_event, cudaEventDisableTiming));
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->world_bytes + w->device_bytes > s->cfg.memory_budget_bytes) {
        cudaEventDestroy(we->edit_event);
        return set_error(VRT_EBUDGET, "world of %llu bytes exceeds the memory budget",
                         (unsigned long long)w->device_bytes);
    }
    s->worlds.push_back(std::move(we));
    s->world_bytes += w->device_bytes;
    *id = (int32_t)s->worlds.size() - 1;
    return VRT_OK;
}

int vrt_server_submit(vrt_server* s, const vrt_request* req) {
    if (!s || !req) return set_error(VRT_EINVAL, "NULL argument");
    Queued q;
    q.req = *req;
    q.submit_ms = s->now();
    q.bytes = 0;
    std::lock_guard<std::mutex> lk(s->mu);
    if (req->world_id < 0 || req->world_id >= (int)s->worlds.size())
        return set_error(VRT_ENOTFOUND, "unknown world %d", req->world_id);
    if (req->kind == VRT_REQ_RENDER) {
        if (req->width < 1 || req->height < 1 || req->width > 32768 || req->height > 32768)
            return set_error(VRT_EINVAL, "bad image size");
        q.bytes = (uint64_t)req->width * req->height * 4;
        if (q.bytes + s->world_bytes > s->cfg.memory_budget_bytes) {
            vrt_completion c{};
            c.user_tag = req->user_tag;
            c.status = VRT_EBUDGET;
            c.kind = req->kind;
            c.submit_ms = c.start_ms = c.done_ms = q.submit_ms;
            s->done.push_back(c);
            return VRT_OK;
        }
    } else if (req->kind != VRT_REQ_EDIT) {
        return set_error(VRT_EINVAL, "unknown request kind %d", req->kind);
    } else if (req->radius < 0 || req->radius > 1024) {
        return set_error(VRT_ERANGE, "edit radius %d", req->radius);
    }
    s->queue.push_back(q);
    return VRT_OK;
}

int vrt_server_poll(vrt_server* s, vrt_completion* out, int32_t max_out) {
    if (!s) return set_error(VRT_EINVAL, "NULL server");
    for (auto& sl : s->slots) {
        if (!sl.busy) continue;
        cudaError_t e = cudaEventQuery(sl.done);
        if (e == cudaSuccess) retire(s, sl);
        else if (e != cudaErrorNotReady) return cuda_error(e, "slot event");
    }
    for (size_t i = 0; i < s->slots.size(); i++) {
        if (s->slots[i].busy) continue;
        int st = VRT_OK;
        if (!admit(s, (int)i, &st)) {
            if (st) return st;
            break;
        }
    }
    int n = 0;
    if (out && max_out > 0) {
        std::lock_guard<std::mutex> lk(s->mu);
        n = (int)std::min<size_t>((size_t)max_out, s->done.size());
        std::copy(s->done.begin(), s->done.begin() + n, out);
        s->done.erase(s->done.begin(), s->done.begin() + n);
    }
    return n;
}

int vrt_server_drain(vrt_server* s) {
    if (!s) return set_error(VRT_EINVAL, "NULL server");
    while (true) {
        int st = vrt_server_poll(s, nullptr, 0);
        if (st < 0) return st;
        bool busy = false;
        for (auto& sl : s->slots) busy |= sl.busy;
        bool queued;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            queued = !s->queue.empty();
        }
        if (!busy && !queued) return VRT_OK;
        if (busy) {
            // wait for the oldest launch instead of spinning
            for (auto& sl : s->slots)
                if (sl.busy) {
                    VRT_CUDA(cudaEventSynchronize(sl.done));
                    break;
                }
        }
    }
}

int vrt_server_wait(vrt_server* s, int32_t timeout_us) {
    if (!s) return set_error(VRT_EINVAL, "NULL server");
    const Clock::time_point end = Clock::now() + std::chrono::microseconds(std::max(0, timeout_us));
    for (;;) {
        bool busy = false;
        for (auto& sl : s->slots) {
            if (!sl.busy) continue;
            busy = true;
            const cudaError_t e = cudaEventQuery(sl.done);
            if (e == cudaSuccess) return 1;
            if (e != cudaErrorNotReady) return cuda_error(e, "slot event");
        }
        if (!busy || Clock::now() >= end) return 0;
        std::this_thread::yield();
    }
}

double vrt_server_now_ms(const vrt_server* s) { return s ? s->now() : 0.0; }

}  // extern "C"
