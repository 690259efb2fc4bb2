// euc_server.cu — the serving loop of the C ABI (euc_server_*).
//
// Resident meshes and textures, a device arena of `framebuffer_budget` bytes
// from which every admitted request takes one block for its targets, and a
// serving thread that forms batches whenever a slot (stream + euc_ctx) is
// free.  A batch is: one fill launch that clears every target of its
// requests, one euc_render_batch per pass index, one device-to-host copy per
// readback target, then a host function on the stream that completes the
// requests and returns their blocks to the arena.  Nothing here renders: the
// images come from euc_render_batch, so they are byte-identical to euc_render
// of the same passes.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/euc_gb300.h"

namespace eucg {
// scene validation of the render path (euc_capi.cu), shared so that a
// request is refused at submission rather than failing its whole batch
int check_scene(const euc_scene *s);
}  // namespace eucg

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint64_t kAlign = 256;

uint32_t bpp_of(uint32_t f) {
    switch (f) {
    case EUC_FMT_RGBA8: case EUC_FMT_BGRA8: case EUC_FMT_R32F: return 4;
    case EUC_FMT_RGB8: return 3;
    default: return 0;  // f32 colour targets are not served (the fill writes 3- or 4-byte texels)
    }
}

uint64_t pad(uint64_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// One target to clear: `bytes` bytes at `p` (256-byte aligned) repeating the
// little-endian texel `pattern` of `period` (3 or 4) bytes.
struct FillDesc {
    unsigned char *p;
    uint64_t bytes;
    uint32_t pattern;
    uint32_t period;
};

// blockIdx.y: the target; the x blocks stride its bytes.
__global__ void __launch_bounds__(256) k_fill(const FillDesc *__restrict__ d) {
    const FillDesc f = d[blockIdx.y];
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f.period == 3) {
        for (uint64_t i = t0; i < f.bytes; i += stride) f.p[i] = (unsigned char)(f.pattern >> (8 * (uint32_t)(i % 3)));
        return;
    }
    const uint4 v = make_uint4(f.pattern, f.pattern, f.pattern, f.pattern);
    const uint64_t nv = f.bytes / 16;
    uint4 *q = reinterpret_cast<uint4 *>(f.p);
    for (uint64_t i = t0; i < nv; i += stride) q[i] = v;
    for (uint64_t i = nv * 16 + t0; i < f.bytes; i += stride) f.p[i] = (unsigned char)(f.pattern >> (8 * (uint32_t)(i & 3)));
}

struct Mesh {
    euc_vertex_layout layout;
    void *verts = nullptr;
    uint64_t nverts = 0;
    uint32_t *idx = nullptr;
    uint64_t nidx = 0;
};

struct Texture {
    void *data = nullptr;
    uint32_t width = 0, height = 0, format = 0;
};

struct PassCopy {
    euc_server_pass p;
    std::vector<unsigned char> uni;
    std::vector<euc_server_binding> binds;
};

struct Req {
    uint64_t id = 0, tag = 0, arrival = 0, admit = 0;
    void *out = nullptr;
    std::vector<euc_server_target> targets;
    std::vector<uint64_t> toff;  // target offsets inside the request's block
    std::vector<PassCopy> passes;
    uint64_t bytes = 0;          // block size
    uint64_t base = 0;           // block offset in the arena
};

// First-fit allocator over [0, size) with coalescing free list.
struct Arena {
    std::map<uint64_t, uint64_t> free_;  // offset -> length
    uint64_t size = 0, used = 0, peak = 0;

    void init(uint64_t n) {
        size = n;
        free_.clear();
        if (n) free_[0] = n;
    }
    bool alloc(uint64_t n, uint64_t *off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            *off = it->first;
            const uint64_t rest = it->second - n, at = it->first + n;
            free_.erase(it);
            if (rest) free_[at] = rest;
            used += n;
            peak = std::max(peak, used);
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t n) {
        used -= n;
        auto next = free_.lower_bound(off);
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                off = prev->first;
                n += prev->second;
                free_.erase(prev);
            }
        }
        if (next != free_.end() && off + n == next->first) {
            n += next->second;
            free_.erase(next);
        }
        free_[off] = n;
    }
};

struct Slot {
    euc_server *srv = nullptr;
    cudaStream_t st = nullptr;
    euc_ctx *ctx = nullptr;
    FillDesc *fill_host = nullptr;  // pinned
    FillDesc *fill_dev = nullptr;
    std::vector<Req *> reqs;
    bool busy = false;
    int status = EUC_OK;
    std::atomic<uint64_t> fill_launches{0};  // written by the serving thread
};

}  // namespace

struct euc_server {
    euc_server_config cfg{};
    unsigned char *arena_dev = nullptr;
    Arena arena;
    Clock::time_point t0;
    std::mutex res_mu;  // meshes, textures
    std::deque<Mesh> meshes;
    std::deque<Texture> textures;
    std::unique_ptr<Slot[]> slots;
    std::mutex mu;  // everything below
    std::condition_variable cv_work, cv_done;
    std::deque<Req *> pending;
    std::deque<euc_server_completion> done;
    uint64_t next_id = 1;
    euc_server_stats stats{};
    bool stop = false;
    std::thread th;
};

namespace {

uint64_t now_ns(const euc_server *s) {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - s->t0).count();
}

// Completes the requests of a slot's batch (mu held).
void finish_slot(euc_server *s, Slot *sl, int status) {
    const uint64_t t = now_ns(s);
    const uint32_t nb = (uint32_t)sl->reqs.size();
    for (Req *r : sl->reqs) {
        euc_server_completion c{};
        c.id = r->id;
        c.tag = r->tag;
        c.status = status;
        c.batch_size = nb;
        c.arrival_ns = r->arrival;
        c.admit_ns = r->admit;
        c.done_ns = t;
        s->done.push_back(c);
        s->arena.release(r->base, r->bytes);
        delete r;
    }
    s->stats.in_flight -= nb;
    s->stats.completed += status == EUC_OK ? nb : 0;
    s->stats.failed += status == EUC_OK ? 0 : nb;
    sl->reqs.clear();
    sl->busy = false;
    s->cv_work.notify_all();
    s->cv_done.notify_all();
}

void CUDART_CB on_batch_done(void *arg) {
    Slot *sl = static_cast<Slot *>(arg);
    euc_server *s = sl->srv;
    std::lock_guard<std::mutex> g(s->mu);
    finish_slot(s, sl, sl->status);
}

euc_target target_of(const euc_server *s, const Req *r, int32_t k) {
    euc_target t{};
    if (k < 0) return t;
    const euc_server_target &st = r->targets[k];
    t.data = s->arena_dev + r->base + r->toff[k];
    t.width = st.width;
    t.height = st.height;
    t.pitch = st.width * bpp_of(st.format);
    t.format = st.format;
    return t;
}

// Host side of one batch: the scenes of every pass index (uniforms patched
// with the bound textures and targets) and the fills.  res_mu held.
void build_batch(const euc_server *s, Slot *sl, std::vector<std::vector<euc_scene>> &scenes,
                 std::vector<FillDesc> &fills) {
    scenes.clear();
    fills.clear();
    for (Req *r : sl->reqs) {
        for (size_t k = 0; k < r->targets.size(); ++k) {
            const euc_server_target &t = r->targets[k];
            const uint32_t bpp = bpp_of(t.format);
            FillDesc f;
            f.p = s->arena_dev + r->base + r->toff[k];
            f.bytes = (uint64_t)t.width * t.height * bpp;
            f.pattern = bpp == 3 ? (t.clear & 0xFFFFFFu) : t.clear;
            f.period = bpp;
            fills.push_back(f);
        }
        for (size_t k = 0; k < r->passes.size(); ++k) {
            if (scenes.size() <= k) scenes.resize(k + 1);
            PassCopy &pc = r->passes[k];
            const Mesh &m = s->meshes[pc.p.mesh];
            for (const euc_server_binding &b : pc.binds) {
                euc_sampler *smp = reinterpret_cast<euc_sampler *>(pc.uni.data() + b.offset);
                if (b.texture >= 0) {
                    const Texture &tx = s->textures[b.texture];
                    smp->data = tx.data;
                    smp->width = tx.width;
                    smp->height = tx.height;
                    smp->pitch = tx.width * 4;
                    smp->format = tx.format;
                } else {
                    const euc_target t = target_of(s, r, b.target);
                    smp->data = t.data;
                    smp->width = t.width;
                    smp->height = t.height;
                    smp->pitch = t.pitch;
                    smp->format = t.format;
                }
            }
            euc_scene sc{};
            sc.desc = pc.p.desc;
            sc.layout = m.layout;
            sc.vertices = m.verts;
            sc.nverts = m.nverts;
            sc.indices = m.idx;
            sc.nindices = m.nidx;
            sc.pixel = target_of(s, r, pc.p.pixel_target);
            sc.depth = target_of(s, r, pc.p.depth_target);
            sc.uniforms = pc.uni.data();
            sc.uniforms_size = pc.uni.size();
            scenes[k].push_back(sc);
        }
    }
}

// Device side of one batch (no lock held).  Returns the first failure; the
// completion host function is enqueued only on success.
int launch_batch(euc_server *s, Slot *sl, const std::vector<std::vector<euc_scene>> &scenes,
                 const std::vector<FillDesc> &fills) {
    const cudaStream_t st = sl->st;
    if (!fills.empty()) {
        std::memcpy(sl->fill_host, fills.data(), fills.size() * sizeof(FillDesc));
        if (cudaMemcpyAsync(sl->fill_dev, sl->fill_host, fills.size() * sizeof(FillDesc), cudaMemcpyHostToDevice, st) !=
            cudaSuccess)
            return EUC_ERR_CUDA;
        k_fill<<<dim3(32, (unsigned)fills.size()), 256, 0, st>>>(sl->fill_dev);
        if (cudaGetLastError() != cudaSuccess) return EUC_ERR_CUDA;
        sl->fill_launches += 1;
    }
    for (const auto &v : scenes)
        if (!v.empty())
            if (int rc = euc_render_batch(sl->ctx, v.data(), v.size(), st)) return rc;
    for (Req *r : sl->reqs) {
        unsigned char *dst = static_cast<unsigned char *>(r->out);
        for (size_t k = 0; k < r->targets.size(); ++k) {
            const euc_server_target &t = r->targets[k];
            if (!t.readback) continue;
            const uint64_t n = (uint64_t)t.width * t.height * bpp_of(t.format);
            if (cudaMemcpyAsync(dst, s->arena_dev + r->base + r->toff[k], n, cudaMemcpyDeviceToHost, st) != cudaSuccess)
                return EUC_ERR_CUDA;
            dst += n;
        }
    }
    if (cudaLaunchHostFunc(st, on_batch_done, sl) != cudaSuccess) return EUC_ERR_CUDA;
    return EUC_OK;
}

void serve(euc_server *s) {
    cudaSetDevice(s->cfg.device);
    std::vector<std::vector<euc_scene>> scenes;
    std::vector<FillDesc> fills;
    std::unique_lock<std::mutex> lk(s->mu);
    while (!s->stop) {
        Slot *sl = nullptr;
        for (uint32_t i = 0; i < s->cfg.slots && !sl; ++i)
            if (!s->slots[i].busy) sl = &s->slots[i];
        uint64_t wake_at = 0;  // 0: wait for a notification
        if (sl && !s->pending.empty()) {
            const uint64_t now = now_ns(s);
            while (!s->pending.empty() && sl->reqs.size() < s->cfg.max_batch) {
                Req *r = s->pending.front();
                if (r->arrival > now) {
                    if (sl->reqs.empty()) wake_at = r->arrival;
                    break;
                }
                if (!s->arena.alloc(r->bytes, &r->base)) break;  // waits for a completion
                r->admit = now;
                s->pending.pop_front();
                sl->reqs.push_back(r);
            }
            if (!sl->reqs.empty()) {
                const uint64_t n = sl->reqs.size();
                sl->busy = true;
                sl->status = EUC_OK;
                s->stats.pending -= n;
                s->stats.in_flight += n;
                s->stats.batches += 1;
                s->stats.batched_requests += n;
                {
                    std::lock_guard<std::mutex> rg(s->res_mu);
                    build_batch(s, sl, scenes, fills);
                }
                lk.unlock();
                const int rc = launch_batch(s, sl, scenes, fills);
                if (rc != EUC_OK) cudaStreamSynchronize(sl->st);  // whatever was enqueued ends first
                lk.lock();
                if (rc != EUC_OK) {
                    (void)cudaGetLastError();
                    finish_slot(s, sl, rc);
                }
                continue;
            }
        }
        if (wake_at)
            s->cv_work.wait_until(lk, s->t0 + std::chrono::nanoseconds(wake_at));
        else
            s->cv_work.wait(lk);
    }
}

void destroy_server(euc_server *s) {
    if (s->slots) {
        for (uint32_t i = 0; i < s->cfg.slots; ++i) {
            Slot &sl = s->slots[i];
            if (sl.st) cudaStreamDestroy(sl.st);
            if (sl.ctx) euc_ctx_destroy(sl.ctx);
            if (sl.fill_host) cudaFreeHost(sl.fill_host);
            if (sl.fill_dev) cudaFree(sl.fill_dev);
        }
    }
    for (Mesh &m : s->meshes) {
        if (m.verts) cudaFree(m.verts);
        if (m.idx) cudaFree(m.idx);
    }
    for (Texture &t : s->textures)
        if (t.data) cudaFree(t.data);
    for (Req *r : s->pending) delete r;
    if (s->arena_dev) cudaFree(s->arena_dev);
    delete s;
}

// Checks one request and copies it (res_mu held).
int check_request(euc_server *s, const euc_server_request &q, Req *&out) {
    out = nullptr;
    if (q.ntargets < 1 || q.ntargets > EUC_SERVER_MAX_TARGETS || !q.targets) return EUC_ERR_INVALID;
    if (q.npasses < 1 || q.npasses > EUC_SERVER_MAX_PASSES || !q.passes) return EUC_ERR_INVALID;
    std::unique_ptr<Req> r(new (std::nothrow) Req());
    if (!r) return EUC_ERR_OOM;
    r->tag = q.tag;
    r->out = q.out;
    uint64_t readback = 0;
    for (uint32_t k = 0; k < q.ntargets; ++k) {
        const euc_server_target &t = q.targets[k];
        const uint32_t bpp = bpp_of(t.format);
        if (!bpp || t.width < 1 || t.height < 1) return EUC_ERR_INVALID;
        if ((uint64_t)t.width * t.height >= 0xFFFFFF00ull) return EUC_ERR_CAPACITY;
        const uint64_t n = (uint64_t)t.width * t.height * bpp;
        r->targets.push_back(t);
        r->toff.push_back(r->bytes);
        r->bytes += pad(n);
        if (t.readback) readback += n;
    }
    if (r->bytes > s->cfg.framebuffer_budget) return EUC_ERR_BUDGET;
    if (readback && (!q.out || q.out_size < readback)) return EUC_ERR_INVALID;
    // a dummy, aligned, non-null device address for the checks of the render path
    unsigned char *const fake = reinterpret_cast<unsigned char *>(kAlign);
    for (uint32_t k = 0; k < q.npasses; ++k) {
        const euc_server_pass &p = q.passes[k];
        if (p.mesh >= s->meshes.size()) return EUC_ERR_INVALID;
        if (p.pixel_target < -1 || p.pixel_target >= (int32_t)q.ntargets) return EUC_ERR_INVALID;
        if (p.depth_target < -1 || p.depth_target >= (int32_t)q.ntargets) return EUC_ERR_INVALID;
        if (p.pixel_target >= 0 && p.pixel_target == p.depth_target) return EUC_ERR_INVALID;
        if (!p.uniforms || p.uniforms_size == 0 || p.uniforms_size > 4096) return EUC_ERR_INVALID;
        if (p.nbindings && !p.bindings) return EUC_ERR_INVALID;
        PassCopy pc;
        pc.p = p;
        pc.uni.assign(static_cast<const unsigned char *>(p.uniforms),
                      static_cast<const unsigned char *>(p.uniforms) + p.uniforms_size);
        pc.binds.assign(p.bindings, p.bindings + p.nbindings);
        pc.p.bindings = nullptr;
        pc.p.uniforms = nullptr;
        std::vector<unsigned char> probe = pc.uni;
        for (const euc_server_binding &b : pc.binds) {
            if ((b.offset & 7) || (uint64_t)b.offset + sizeof(euc_sampler) > p.uniforms_size) return EUC_ERR_INVALID;
            if ((b.texture >= 0) == (b.target >= 0)) return EUC_ERR_INVALID;  // exactly one source
            euc_sampler *smp = reinterpret_cast<euc_sampler *>(probe.data() + b.offset);
            if (b.texture >= 0) {
                if ((uint64_t)b.texture >= s->textures.size()) return EUC_ERR_INVALID;
                const Texture &tx = s->textures[b.texture];
                smp->width = tx.width;
                smp->height = tx.height;
                smp->pitch = tx.width * 4;
                smp->format = tx.format;
            } else {
                if (b.target >= (int32_t)q.ntargets) return EUC_ERR_INVALID;
                // read-only in this pass; formats a sampler reads
                if (b.target == p.pixel_target || b.target == p.depth_target) return EUC_ERR_INVALID;
                const euc_server_target &t = q.targets[b.target];
                if (t.format != EUC_FMT_RGBA8 && t.format != EUC_FMT_R32F) return EUC_ERR_INVALID;
                smp->width = t.width;
                smp->height = t.height;
                smp->pitch = t.width * 4;
                smp->format = t.format;
            }
            smp->data = fake;
        }
        const Mesh &m = s->meshes[p.mesh];
        euc_scene sc{};
        sc.desc = p.desc;
        sc.layout = m.layout;
        sc.vertices = m.verts;
        sc.nverts = m.nverts;
        sc.indices = m.idx;
        sc.nindices = m.nidx;
        auto tgt = [&](int32_t i) {
            euc_target t{};
            if (i < 0) return t;
            const euc_server_target &st = q.targets[i];
            t.data = fake;
            t.width = st.width;
            t.height = st.height;
            t.pitch = st.width * bpp_of(st.format);
            t.format = st.format;
            return t;
        };
        sc.pixel = tgt(p.pixel_target);
        sc.depth = tgt(p.depth_target);
        sc.uniforms = probe.data();
        sc.uniforms_size = probe.size();
        if (int rc = eucg::check_scene(&sc)) return rc;
        r->passes.push_back(std::move(pc));
    }
    out = r.release();
    return EUC_OK;
}

}  // namespace

extern "C" {

int euc_server_create(const euc_server_config *config, euc_server **out) {
    if (!config || !out) return EUC_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess) {
        (void)cudaGetLastError();
        return EUC_ERR_CUDA;
    }
    if (config->device < 0 || config->device >= ndev || config->framebuffer_budget == 0) return EUC_ERR_INVALID;
    if (config->slots > 16 || config->max_batch > 4096) return EUC_ERR_INVALID;
    if (cudaSetDevice(config->device) != cudaSuccess) return EUC_ERR_CUDA;
    euc_server *s = new (std::nothrow) euc_server();
    if (!s) return EUC_ERR_OOM;
    s->cfg = *config;
    if (!s->cfg.max_batch) s->cfg.max_batch = 256;
    if (!s->cfg.slots) s->cfg.slots = 3;
    if (!s->cfg.max_pending) s->cfg.max_pending = 1u << 20;
    s->cfg.framebuffer_budget = pad(s->cfg.framebuffer_budget);
    s->t0 = Clock::now();
    int rc = EUC_OK;
    if (cudaMalloc(&s->arena_dev, s->cfg.framebuffer_budget) != cudaSuccess) rc = EUC_ERR_OOM;
    s->arena.init(s->cfg.framebuffer_budget);
    s->stats.budget_bytes = s->cfg.framebuffer_budget;
    s->slots.reset(new (std::nothrow) Slot[s->cfg.slots]);
    if (!s->slots) rc = EUC_ERR_OOM;
    const size_t fbytes = (size_t)s->cfg.max_batch * EUC_SERVER_MAX_TARGETS * sizeof(FillDesc);
    for (uint32_t i = 0; rc == EUC_OK && i < s->cfg.slots; ++i) {
        Slot &sl = s->slots[i];
        sl.srv = s;
        if (cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking) != cudaSuccess) rc = EUC_ERR_CUDA;
        else if (cudaMallocHost(&sl.fill_host, fbytes) != cudaSuccess || cudaMalloc(&sl.fill_dev, fbytes) != cudaSuccess)
            rc = EUC_ERR_OOM;
        else rc = euc_ctx_create(config->device, &sl.ctx);
    }
    if (rc != EUC_OK) {
        (void)cudaGetLastError();
        destroy_server(s);
        return rc;
    }
    try {
        s->th = std::thread(serve, s);
    } catch (...) {
        destroy_server(s);
        return EUC_ERR_OOM;
    }
    *out = s;
    return EUC_OK;
}

int euc_server_destroy(euc_server *s) {
    if (!s) return EUC_ERR_INVALID;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->th.joinable()) s->th.join();
    cudaSetDevice(s->cfg.device);
    for (uint32_t i = 0; i < s->cfg.slots; ++i)
        if (s->slots[i].st) cudaStreamSynchronize(s->slots[i].st);  // their host functions complete the batches
    destroy_server(s);
    return EUC_OK;
}

int euc_server_add_mesh(euc_server *s, const euc_vertex_layout *layout, const void *vertices, size_t nverts,
                        const uint32_t *indices, size_t nindices, uint32_t *id) {
    if (!s || !layout || !id || (nverts && !vertices) || (nindices && !indices)) return EUC_ERR_INVALID;
    if (layout->stride == 0 || (layout->stride & 3) || nverts >= 0xFFFFFFFFull) return EUC_ERR_INVALID;
    // index bounds are checked here, once, so that no batch meets them on the device
    for (size_t i = 0; i < nindices; ++i)
        if (indices[i] >= nverts) return EUC_ERR_INDEX_OOB;
    Mesh m;
    m.layout = *layout;
    m.nverts = nverts;
    m.nidx = indices ? nindices : 0;
    if (cudaSetDevice(s->cfg.device) != cudaSuccess) return EUC_ERR_CUDA;
    const size_t vb = nverts * layout->stride;
    if (vb && (cudaMalloc(&m.verts, vb) != cudaSuccess ||
               cudaMemcpy(m.verts, vertices, vb, cudaMemcpyHostToDevice) != cudaSuccess)) {
        (void)cudaGetLastError();
        if (m.verts) cudaFree(m.verts);
        return EUC_ERR_OOM;
    }
    if (indices && (cudaMalloc(&m.idx, std::max<size_t>(nindices, 1) * 4) != cudaSuccess ||
                    cudaMemcpy(m.idx, indices, nindices * 4, cudaMemcpyHostToDevice) != cudaSuccess)) {
        (void)cudaGetLastError();
        if (m.verts) cudaFree(m.verts);
        if (m.idx) cudaFree(m.idx);
        return EUC_ERR_OOM;
    }
    std::lock_guard<std::mutex> g(s->res_mu);
    *id = (uint32_t)s->meshes.size();
    s->meshes.push_back(m);
    return EUC_OK;
}

int euc_server_add_texture(euc_server *s, const void *texels, uint32_t width, uint32_t height, uint64_t pitch,
                           uint32_t format, uint32_t *id) {
    if (!s || !texels || !id || width < 1 || height < 1) return EUC_ERR_INVALID;
    if (format != EUC_FMT_RGBA8 && format != EUC_FMT_R32F) return EUC_ERR_INVALID;
    const uint64_t row = (uint64_t)width * 4;
    if (!pitch) pitch = row;
    if (pitch < row) return EUC_ERR_INVALID;
    Texture t;
    t.width = width;
    t.height = height;
    t.format = format;
    if (cudaSetDevice(s->cfg.device) != cudaSuccess) return EUC_ERR_CUDA;
    if (cudaMalloc(&t.data, row * height) != cudaSuccess ||
        cudaMemcpy2D(t.data, row, texels, pitch, row, height, cudaMemcpyHostToDevice) != cudaSuccess) {
        (void)cudaGetLastError();
        if (t.data) cudaFree(t.data);
        return EUC_ERR_OOM;
    }
    std::lock_guard<std::mutex> g(s->res_mu);
    *id = (uint32_t)s->textures.size();
    s->textures.push_back(t);
    return EUC_OK;
}

uint64_t euc_server_now_ns(euc_server *s) { return s ? now_ns(s) : 0; }

int euc_server_submit(euc_server *s, const euc_server_request *reqs, size_t n, uint64_t *first_id, size_t *accepted) {
    if (accepted) *accepted = 0;
    if (!s || (n && !reqs)) return EUC_ERR_INVALID;
    std::vector<Req *> copies;
    copies.reserve(n);
    int rc = EUC_OK;
    {
        std::lock_guard<std::mutex> g(s->res_mu);
        for (size_t i = 0; i < n && rc == EUC_OK; ++i) {
            Req *r = nullptr;
            rc = check_request(s, reqs[i], r);
            if (rc == EUC_OK) copies.push_back(r);
        }
    }
    if (rc != EUC_OK) {
        for (Req *r : copies) delete r;
        return rc;
    }
    std::lock_guard<std::mutex> g(s->mu);
    const uint64_t now = now_ns(s);
    size_t k = 0;
    if (first_id) *first_id = s->next_id;
    for (; k < copies.size(); ++k) {
        if (s->stats.pending >= s->cfg.max_pending) break;
        Req *r = copies[k];
        r->id = s->next_id++;
        r->arrival = reqs[k].arrival_ns ? reqs[k].arrival_ns : now;
        s->pending.push_back(r);
        s->stats.pending += 1;
    }
    s->stats.submitted += k;
    s->stats.refused += copies.size() - k;
    for (size_t j = k; j < copies.size(); ++j) delete copies[j];
    if (accepted) *accepted = k;
    if (k) s->cv_work.notify_all();
    return k == copies.size() ? EUC_OK : EUC_ERR_BUSY;
}

int euc_server_poll(euc_server *s, euc_server_completion *out, size_t max, size_t *n, int wait_ms) {
    if (!s || !n || (max && !out)) return EUC_ERR_INVALID;
    *n = 0;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->done.empty() && wait_ms > 0)
        s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty(); });
    size_t k = 0;
    while (k < max && !s->done.empty()) {
        out[k++] = s->done.front();
        s->done.pop_front();
    }
    *n = k;
    return EUC_OK;
}

int euc_server_drain(euc_server *s, int timeout_ms) {
    if (!s) return EUC_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto idle = [&] { return s->stats.pending == 0 && s->stats.in_flight == 0; };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, idle);
        return EUC_OK;
    }
    return s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), idle) ? EUC_OK : EUC_ERR_TIMEOUT;
}

int euc_server_stats_get(euc_server *s, euc_server_stats *out) {
    if (!s || !out) return EUC_ERR_INVALID;
    // render launches: each slot context counts its own (and resets on read)
    uint64_t renders = 0;
    for (uint32_t i = 0; i < s->cfg.slots; ++i) {
        uint64_t n = 0;
        if (euc_ctx_profile(s->slots[i].ctx, nullptr, &n) == EUC_OK) renders += n;
    }
    std::lock_guard<std::mutex> g(s->mu);
    s->stats.launches += renders;
    *out = s->stats;
    out->budget_used = s->arena.used;
    out->budget_peak = s->arena.peak;
    uint64_t fills = 0;
    for (uint32_t i = 0; i < s->cfg.slots; ++i) fills += s->slots[i].fill_launches.load();
    out->launches += fills;
    return EUC_OK;
}

}  // extern "C"
