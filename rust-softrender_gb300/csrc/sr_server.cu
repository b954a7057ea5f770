// sr_server.cu — the serving loop (continuous batching) over sr_batch.
//
// A worker thread makes every rendering call of the server (the copies of a
// result run on the thread that reads it).  Submitted requests
// wait in a FIFO; whenever a batch slot is free and the head of the FIFO fits
// the HBM budget, the worker takes every queued request that fits (up to
// max_batch, in arrival order) and renders them as one batch on that slot's
// stream.  Up to max_inflight batches run on the GPU at once, so requests that
// arrive while earlier batches execute are admitted as slots and memory free
// up and their work overlaps with the earlier batches.  A host function on the
// slot's stream stamps the completion time of its requests.
//
// Targets (pipelines: colour, depth, per-pixel keys) are pooled by size and
// format and stay resident until the caller reads or releases the result;
// the pool then keeps them for reuse.  Pooled targets count against the HBM
// budget with the admitted requests, and are freed when admitted work needs
// their room.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <iterator>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "sr_host.h"

using namespace sr;

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    uint64_t ticket;
    sr_request r;
    sr_uniforms U;
    uint64_t bytes;             // admitted footprint
    Clock::time_point t_submit, t_done;
    sr_pipeline* target = nullptr;
    bool done = false;
    int status = SR_OK;
};

struct Slot {
    sr_batch* batch = nullptr;
    cudaStream_t stream = nullptr;
    bool busy = false;
    std::vector<Req*> reqs;     // the batch on the GPU
};

// Pooled targets come in pixel-capacity classes (powers of two), so that any
// frame of a class can reuse any pooled target of that class and format.
uint64_t px_class(uint32_t w, uint32_t h) {
    uint64_t c = 4096;
    while (c < (uint64_t)w * h) c <<= 1;
    return c;
}

// Device bytes of a pooled target of pixel class `px`: colour, depth and
// per-pixel keys, the touched-block bitmap, flags.
uint64_t class_bytes(uint64_t px, uint32_t fmt) {
    return px * ((fmt == SR_COLOR_RGBA32F ? 16 : 4) + 4 + 8) + px / 256 + 4096;
}

uint64_t target_bytes(uint32_t w, uint32_t h, uint32_t fmt) { return class_bytes(px_class(w, h), fmt); }

uint64_t request_bytes(const sr_request& r) {
    const sr_mesh* m = r.draw.mesh;
    // the target plus this request's share of the batch scratch
    return target_bytes(r.width, r.height, r.color_format) + (uint64_t)(m->n_indices / 3) * 96 +
           (uint64_t)m->n_pad * 64;
}

}  // namespace

struct sr_server {
    sr_server_config cfg;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Req*> pending;
    std::unordered_map<uint64_t, Req*> reqs;
    std::vector<Slot> slots;
    std::multimap<std::pair<uint64_t, uint32_t>, sr_pipeline*> pool;   // (pixel class, format)
    uint64_t next_ticket = 1;
    uint64_t in_use = 0, peak = 0;
    uint64_t pool_bytes = 0;    // targets held in the pool for reuse
    uint32_t inflight = 0;
    bool stop = false;
    int device = 0;
    std::thread worker;
    // statistics
    std::vector<double> lat_ms;
    uint64_t submitted = 0, batches = 0, batched_reqs = 0;
    Clock::time_point t_first, t_last;
    bool have_first = false;
};

namespace {

struct DoneCtx {
    sr_server* s;
    Slot* slot;
};

// Host function at the end of a slot's batch: stamps its requests.
void CUDART_CB batch_done(void* p) {
    DoneCtx* c = static_cast<DoneCtx*>(p);
    sr_server* s = c->s;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        const Clock::time_point now = Clock::now();
        for (Req* q : c->slot->reqs) {
            q->t_done = now;
            q->done = true;
            s->lat_ms.push_back(std::chrono::duration<double, std::milli>(now - q->t_submit).count());
        }
        s->t_last = now;
        c->slot->reqs.clear();
        c->slot->busy = false;
        --s->inflight;
    }
    s->cv.notify_all();
    delete c;
}

sr_pipeline* take_target(sr_server* s, uint32_t w, uint32_t h, uint32_t fmt) {
    const uint64_t cls = px_class(w, h);
    sr_pipeline* p = nullptr;
    std::vector<sr_pipeline*> evict;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->pool.find(std::make_pair(cls, fmt));
        if (it != s->pool.end()) {
            p = it->second;
            s->pool.erase(it);
            s->pool_bytes -= class_bytes(cls, fmt);
        }
        // the pool counts against the budget too: while the admitted requests
        // and the pooled targets together exceed it, pooled targets go,
        // largest first (fewest frees)
        while (!s->pool.empty() && s->in_use + s->pool_bytes > s->cfg.hbm_budget) {
            const auto e = std::prev(s->pool.end());
            s->pool_bytes -= class_bytes(e->first.first, e->first.second);
            evict.push_back(e->second);
            s->pool.erase(e);
        }
    }
    for (sr_pipeline* e : evict) sr_pipeline_destroy(e);
    if (!p) {
        sr_fb_desc fb{w, h, fmt, 1, 0};
        if (pipeline_create_cap(&fb, cls, &p) != SR_OK) return nullptr;
    }
    if (pipeline_retarget(p, w, h) != SR_OK) { sr_pipeline_destroy(p); return nullptr; }
    return p;
}

void serve_plain(sr_server* s, Req* q) {
    sr_pipeline* p = take_target(s, q->r.width, q->r.height, q->r.color_format);
    int st = p ? SR_OK : SR_ENOMEM;
    if (p) {
        q->target = p;
        sr_pipeline_set_uniforms(p, &q->U, sizeof(sr_uniforms));
        sr_framebuffer_clear(p, q->r.clear_color);
        sr_draw d = q->r.draw;
        st = sr_render(p, &d);
        const int st2 = sr_sync(p);
        if (st == SR_OK && st2 != SR_ENAN) st = st2;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    const Clock::time_point now = Clock::now();
    q->t_done = now;
    q->done = true;
    q->status = st;
    s->lat_ms.push_back(std::chrono::duration<double, std::milli>(now - q->t_submit).count());
    s->t_last = now;
    ++s->batches;
    ++s->batched_reqs;
    --s->inflight;
    s->cv.notify_all();
}

void worker_main(sr_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        std::vector<Req*> take;
        Slot* slot = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait(lk, [&] {
                if (s->stop) return true;
                if (s->pending.empty() || s->inflight >= s->cfg.max_inflight) return false;
                return s->in_use + s->pending.front()->bytes <= s->cfg.hbm_budget;
            });
            if (s->stop) return;
            // admit in arrival order while requests fit the budget
            while (!s->pending.empty() && take.size() < s->cfg.max_batch) {
                Req* q = s->pending.front();
                if (s->in_use + q->bytes > s->cfg.hbm_budget) break;
                s->in_use += q->bytes;
                s->pending.pop_front();
                take.push_back(q);
                if (s->cfg.plain) break;
            }
            s->peak = std::max(s->peak, s->in_use);
            ++s->inflight;
            if (!s->cfg.plain) {
                for (auto& sl : s->slots)
                    if (!sl.busy) { slot = &sl; break; }
                slot->busy = true;
                slot->reqs = take;
                ++s->batches;
                s->batched_reqs += take.size();
            }
        }
        if (s->cfg.plain) {
            serve_plain(s, take[0]);
            continue;
        }
        std::vector<sr_batch_item> items(take.size());
        size_t k = 0;
        for (Req* q : take) {
            sr_pipeline* p = take_target(s, q->r.width, q->r.height, q->r.color_format);
            q->target = p;
            if (!p) { q->status = SR_ENOMEM; continue; }
            sr_pipeline_set_uniforms(p, &q->U, sizeof(sr_uniforms));
            sr_batch_item& it = items[k++];
            std::memset(&it, 0, sizeof(it));
            it.target = p;
            it.draw = q->r.draw;
            it.clear = 1;
            std::memcpy(it.clear_color, q->r.clear_color, 16);
        }
        int st = k ? sr_batch_render(slot->batch, items.data(), (uint32_t)k) : SR_OK;
        if (st != SR_OK)
            for (Req* q : take) q->status = st;
        DoneCtx* c = new DoneCtx{s, slot};
        if (cudaLaunchHostFunc(slot->stream, batch_done, c) != cudaSuccess) {
            cudaStreamSynchronize(slot->stream);
            batch_done(c);
        }
    }
}

}  // namespace

extern "C" SR_API int sr_server_create(const sr_server_config* cfg, sr_server** out) {
    if (!out) return SR_EINVAL;
    *out = nullptr;
    sr_server* s = new (std::nothrow) sr_server();
    if (!s) return SR_ENOMEM;
    std::memset(&s->cfg, 0, sizeof(s->cfg));
    if (cfg) s->cfg = *cfg;
    if (!s->cfg.hbm_budget) s->cfg.hbm_budget = 64ull << 30;
    if (!s->cfg.max_inflight) s->cfg.max_inflight = 3;
    if (!s->cfg.max_batch) s->cfg.max_batch = 256;
    if (s->cfg.max_inflight > 16) s->cfg.max_inflight = 16;
    if (s->cfg.plain) s->cfg.max_inflight = 1;
    cudaGetDevice(&s->device);
    s->slots.resize(s->cfg.plain ? 0 : s->cfg.max_inflight);
    for (auto& sl : s->slots) {
        int rc = sr_batch_create(&sl.batch);
        if (rc == SR_OK && cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess) rc = SR_ECUDA;
        if (rc == SR_OK) rc = sr_batch_set_stream(sl.batch, sl.stream);
        // request latency must not include one-time measurements
        if (rc == SR_OK) rc = sr_batch_set_options(sl.batch, 1, 0);
        if (rc != SR_OK) { sr_server_destroy(s); return rc; }
    }
    s->worker = std::thread(worker_main, s);
    *out = s;
    return SR_OK;
}

extern "C" SR_API int sr_server_submit(sr_server* s, const sr_request* r, uint64_t* ticket) {
    if (!s || !r || !ticket || !r->uniforms || r->uniforms_size != sizeof(sr_uniforms)) return SR_EINVAL;
    const sr_draw* d = &r->draw;
    // everything sr_batch_render checks of the draw alone: a request it would
    // refuse is refused here, not with the batch it was folded into
    const int rc = batch_draw_check(d);
    if (rc != SR_OK) return rc;
    if (r->width == 0 || r->height == 0 || r->width > 32767 || r->height > 32767) return SR_EINVAL;
    if (r->color_format != SR_COLOR_RGBA8 && r->color_format != SR_COLOR_RGBA32F) return SR_EINVAL;
    Req* q = new (std::nothrow) Req();
    if (!q) return SR_ENOMEM;
    q->r = *r;
    std::memcpy(&q->U, r->uniforms, sizeof(sr_uniforms));
    q->r.uniforms = nullptr;
    q->bytes = request_bytes(*r);
    if (q->bytes > s->cfg.hbm_budget) { delete q; return SR_EBUDGET; }
    // the request reads its mesh and texture until it is read or released
    mesh_ref(d->mesh);
    texture_ref(d->texture);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        q->ticket = s->next_ticket++;
        q->t_submit = Clock::now();
        if (!s->have_first) { s->t_first = q->t_submit; s->have_first = true; }
        s->reqs[q->ticket] = q;
        s->pending.push_back(q);
        ++s->submitted;
        *ticket = q->ticket;
    }
    s->cv.notify_all();
    return SR_OK;
}

extern "C" SR_API int sr_server_wait(sr_server* s, uint64_t ticket, uint32_t timeout_ms) {
    if (!s) return SR_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->reqs.find(ticket) == s->reqs.end()) return SR_EINVAL;
    // looked up again on every wake-up: another thread may read (and free)
    // the request meanwhile
    Req* q = nullptr;
    const bool ok = s->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] {
        auto it = s->reqs.find(ticket);
        q = it == s->reqs.end() ? nullptr : it->second;
        return !q || q->done;
    });
    if (!ok) return SR_ETIMEOUT;
    return q ? q->status : SR_EINVAL;
}

namespace {
int finish(sr_server* s, uint64_t ticket, void* color, float* depth) {
    Req* q = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        if (it == s->reqs.end()) return SR_EINVAL;
        q = it->second;
        if (!q->done) return SR_EBUSY;
        s->reqs.erase(it);
    }
    int st = q->status;
    if (q->target && (color || depth) && st == SR_OK) st = sr_framebuffer_read(q->target, color, depth, nullptr);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (q->target) {
            const uint64_t cls = px_class(q->r.width, q->r.height);
            s->pool.emplace(std::make_pair(cls, q->r.color_format), q->target);
            s->pool_bytes += class_bytes(cls, q->r.color_format);
        }
        s->in_use -= q->bytes;
    }
    s->cv.notify_all();
    mesh_unref(q->r.draw.mesh);
    texture_unref(q->r.draw.texture);
    delete q;
    return st == SR_ENAN ? SR_OK : st;
}
}  // namespace

extern "C" SR_API int sr_server_read(sr_server* s, uint64_t ticket, void* color, float* depth) {
    if (!s) return SR_EINVAL;
    return finish(s, ticket, color, depth);
}

extern "C" SR_API int sr_server_release(sr_server* s, uint64_t ticket) {
    if (!s) return SR_EINVAL;
    return finish(s, ticket, nullptr, nullptr);
}

extern "C" SR_API int sr_server_drain(sr_server* s, uint32_t timeout_ms) {
    if (!s) return SR_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] {
        if (!s->pending.empty() || s->inflight) return false;
        for (auto& kv : s->reqs)
            if (!kv.second->done) return false;
        return true;
    });
    return ok ? SR_OK : SR_ETIMEOUT;
}

extern "C" SR_API int sr_server_get_stats(sr_server* s, sr_server_stats* out) {
    if (!s || !out) return SR_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->lat_ms.size();
    out->batches = s->batches;
    out->mean_batch = s->batches ? (double)s->batched_reqs / (double)s->batches : 0.0;
    out->peak_bytes = s->peak;
    if (!s->lat_ms.empty()) {
        std::vector<double> v = s->lat_ms;
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) {
            const size_t i = (size_t)std::min<double>((double)(v.size() - 1), std::ceil(p * v.size()) - 1.0);
            return v[i];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        double sum = 0.0;
        for (double x : v) sum += x;
        out->mean_ms = sum / (double)v.size();
        out->max_ms = v.back();
        const double span = std::chrono::duration<double>(s->t_last - s->t_first).count();
        out->throughput_rps = span > 0.0 ? (double)v.size() / span : 0.0;
    }
    return SR_OK;
}

extern "C" SR_API int sr_server_reset_stats(sr_server* s) {
    if (!s) return SR_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat_ms.clear();
    s->submitted = s->batches = s->batched_reqs = 0;
    s->have_first = false;
    s->peak = s->in_use;
    return SR_OK;
}

extern "C" SR_API int sr_server_destroy(sr_server* s) {
    if (!s) return SR_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (auto& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.batch) sr_batch_destroy(sl.batch);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    for (auto& kv : s->reqs) {
        if (kv.second->target) sr_pipeline_destroy(kv.second->target);
        mesh_unref(kv.second->r.draw.mesh);
        texture_unref(kv.second->r.draw.texture);
        delete kv.second;
    }
    for (auto& kv : s->pool) sr_pipeline_destroy(kv.second);
    delete s;
    return SR_OK;
}
