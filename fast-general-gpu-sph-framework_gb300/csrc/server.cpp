// server.cpp — continuous-batching scene server (host side, over the C ABI).
//
// The reference steps one scene per process and has no serving layer. This
// is the native counterpart of a request loop: requests (a scene's initial
// state and a number of frames) wait in a FIFO queue and are admitted between
// chunks of frames while the resident scenes' device state fits the memory
// budget; each goes to a batch with room for it (capacity: particles, cells,
// scenes), and a new batch is opened while fewer than max_batches are. The
// resident scenes of a batch are stepped together (one launch per stage for
// all of them), the batches on their own streams at once; a chunk stops at
// the earliest completion, so every request is stepped exactly its frames;
// finished requests leave the batch (gsph_batch_repack, together with the
// admissions of the next step) and their final state waits for
// gsph_server_take. A scene's evolution in a batch is bit-identical to its
// evolution alone, so results do not depend on the mix.
//
// Thread-safety: submit / poll / take / stats may be called from other
// threads while gsph_server_step runs; step itself is called by one thread.

#include <algorithm>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <unordered_map>
#include <vector>

#include "gsph_internal.h"

namespace {

void fail(const char *msg) { gsph::set_error("%s", msg); }

// Device bytes a scene holds in a batch: particle state (two buffer sets),
// force, sort and split workspace, neighbour masks and occupied-cell lists
// per particle; cell offsets, slab words and group offsets per cell.
constexpr uint64_t kBytesPerParticle = 221;
constexpr uint64_t kBytesPerCell = 44;

struct Request {
    uint64_t id = 0;
    gsph_params params{};
    std::vector<float> pos, vel;   // float4 per particle
    uint32_t n = 0;
    uint64_t cells = 0;
    uint32_t frames = 0;
    uint32_t remaining = 0;
    uint64_t bytes() const { return kBytesPerParticle * n + kBytesPerCell * cells; }
};

}  // namespace

// One batch handle and the requests resident in it (in batch order). A
// batch's key space holds at most 2^26 cells, so the server opens further
// batches (up to max_batches) rather than let the key space cap residency:
// the memory budget is what bounds the resident scenes.
struct Shard {
    gsph_handle batch = nullptr;
    std::vector<Request> resident;
};

struct gsph_server {
    gsph_server_config cfg{};
    std::vector<Shard> shards;
    std::mutex mu;                       // queue, finished, stats, residents' counters
    std::deque<Request> queue;
    std::deque<uint64_t> finished_order;
    std::unordered_map<uint64_t, Request> finished;
    gsph_server_stats stats{};
};

namespace {

bool fits(const gsph_server_config &cfg, uint64_t n, uint64_t c, uint64_t scenes,
          uint64_t bytes) {
    return bytes <= cfg.budget_bytes && n <= cfg.particle_capacity &&
           c <= cfg.cell_capacity && scenes <= cfg.scene_capacity;
}

uint64_t cells_of(const gsph_params &p) {
    return uint64_t(p.grid_size[0]) * uint64_t(p.grid_size[1]) * uint64_t(p.grid_size[2]);
}

int max_batches(const gsph_server_config &cfg) {
    return cfg.max_batches > 0 ? cfg.max_batches : 1;
}

}  // namespace

extern "C" {

gsph_status gsph_server_create(const gsph_server_config *cfg, gsph_server_handle *out) {
    if (!cfg || !out) {
        fail("gsph_server_create: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    *out = nullptr;
    if (cfg->chunk_frames < 1 || cfg->particle_capacity == 0 || cfg->cell_capacity == 0 ||
        cfg->scene_capacity == 0 || cfg->particle_capacity > 0x7FFFFFFFull ||
        cfg->cell_capacity >= 67108864ull || cfg->max_batches < 0) {
        fail("gsph_server_create: chunk_frames >= 1 and capacities in range needed");
        return GSPH_ERR_INVALID_ARG;
    }
    gsph_server *s = new (std::nothrow) gsph_server();
    if (!s) {
        fail("gsph_server_create: host allocation failed");
        return GSPH_ERR_OUT_OF_MEMORY;
    }
    s->cfg = *cfg;
    *out = s;
    return GSPH_OK;
}

gsph_status gsph_server_destroy(gsph_server_handle s) {
    if (!s) return GSPH_OK;
    for (Shard &sh : s->shards)
        if (sh.batch) gsph_destroy(sh.batch);
    delete s;
    return GSPH_OK;
}

gsph_status gsph_server_submit(gsph_server_handle s, uint64_t id, const gsph_params *p,
                               const float *pos4, const float *vel4, uint32_t n,
                               uint32_t frames) {
    if (!s || !p || (n && !pos4) || frames == 0) {
        fail("gsph_server_submit: null argument or zero frames");
        return GSPH_ERR_INVALID_ARG;
    }
    Request r;
    r.id = id;
    r.params = *p;
    r.n = n;
    r.cells = cells_of(*p);
    r.frames = r.remaining = frames;
    try {
        r.pos.assign(pos4, pos4 + size_t(n) * 4);
        if (vel4) r.vel.assign(vel4, vel4 + size_t(n) * 4);
    } catch (...) {
        fail("gsph_server_submit: host allocation failed");
        return GSPH_ERR_OUT_OF_MEMORY;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    s->queue.push_back(std::move(r));
    ++s->stats.submitted;
    return GSPH_OK;
}

namespace {

// Per-shard totals of the scenes that stay and of the ones admitted now.
struct ShardPlan {
    std::vector<uint32_t> keep;
    std::vector<Request> admitted;
    uint64_t n = 0, c = 0;
};

// Creates or repacks shard `sh` for its plan.
gsph_status apply_plan(const gsph_server_config &cfg, Shard &sh, ShardPlan &pl) {
    std::vector<gsph_params> plist;
    std::vector<uint32_t> counts;
    std::vector<float> pos, vel;
    bool any_vel = false;
    for (const Request &r : pl.admitted) any_vel |= !r.vel.empty();
    for (const Request &r : pl.admitted) {
        plist.push_back(r.params);
        counts.push_back(r.n);
        pos.insert(pos.end(), r.pos.begin(), r.pos.end());
        if (any_vel) {
            if (r.vel.empty())
                vel.insert(vel.end(), size_t(r.n) * 4, 0.f);
            else
                vel.insert(vel.end(), r.vel.begin(), r.vel.end());
        }
    }
    if (!sh.batch)
        return gsph_batch_create_ex(plist.data(), counts.data(), uint32_t(plist.size()),
                                    pos.empty() ? nullptr : pos.data(),
                                    any_vel ? vel.data() : nullptr, cfg.particle_capacity,
                                    cfg.cell_capacity, cfg.scene_capacity, cfg.device,
                                    &sh.batch);
    return gsph_batch_repack(sh.batch, pl.keep.empty() ? nullptr : pl.keep.data(),
                             uint32_t(pl.keep.size()), plist.empty() ? nullptr : plist.data(),
                             counts.empty() ? nullptr : counts.data(), uint32_t(plist.size()),
                             pos.empty() ? nullptr : pos.data(),
                             any_vel ? vel.data() : nullptr);
}

}  // namespace

gsph_status gsph_server_step(gsph_server_handle s, int *frames_stepped) {
    if (!s) {
        fail("gsph_server_step: null server");
        return GSPH_ERR_INVALID_ARG;
    }
    if (frames_stepped) *frames_stepped = 0;
    const gsph_server_config &cfg = s->cfg;
    // 1. retire finished scenes and admit queued requests that fit (FIFO): a
    //    request goes to the first batch with room for it, or to a new batch
    //    while fewer than max_batches are open; the budget bounds the resident
    //    bytes of all batches together
    std::vector<ShardPlan> plan(s->shards.size());
    uint64_t bytes = 0;
    for (size_t b = 0; b < s->shards.size(); ++b) {
        const std::vector<Request> &res = s->shards[b].resident;
        for (size_t k = 0; k < res.size(); ++k) {
            const Request &r = res[k];
            if (r.remaining == 0) continue;
            plan[b].keep.push_back(uint32_t(k));
            plan[b].n += r.n;
            plan[b].c += r.cells;
            bytes += r.bytes();
        }
    }
    {
        std::lock_guard<std::mutex> lock(s->mu);
        for (;;) {
            while (!s->queue.empty()) {
                const Request &h = s->queue.front();
                if (bytes + h.bytes() > cfg.budget_bytes) break;
                size_t b = 0;
                for (; b < plan.size(); ++b) {
                    const ShardPlan &pl = plan[b];
                    const uint64_t scenes = pl.keep.size() + pl.admitted.size() + 1;
                    if (fits(cfg, pl.n + h.n, pl.c + h.cells, scenes, 0)) break;
                }
                if (b == plan.size()) {
                    // a new batch, if one may be opened and the head fits it
                    if (int(plan.size()) >= max_batches(cfg) ||
                        !fits(cfg, h.n, h.cells, 1, 0))
                        break;
                    plan.emplace_back();
                }
                ShardPlan &pl = plan[b];
                pl.n += h.n;
                pl.c += h.cells;
                bytes += h.bytes();
                pl.admitted.push_back(std::move(s->queue.front()));
                s->queue.pop_front();
            }
            // a head that cannot fit even alone would block the queue forever
            if (!s->queue.empty()) {
                const Request &h = s->queue.front();
                if (!fits(cfg, h.n, h.cells, 1, h.bytes())) {
                    s->queue.pop_front();
                    ++s->stats.rejected;
                    continue;
                }
            }
            break;
        }
    }
    if (plan.size() > s->shards.size()) {
        std::lock_guard<std::mutex> lock(s->mu);   // get_stats walks the shards
        s->shards.resize(plan.size());
    }
    for (size_t b = 0; b < plan.size(); ++b) {
        Shard &sh = s->shards[b];
        ShardPlan &pl = plan[b];
        const bool changed = !pl.admitted.empty() || pl.keep.size() != sh.resident.size();
        if (!changed) continue;
        gsph_status st = (sh.batch || !pl.admitted.empty()) ? apply_plan(cfg, sh, pl)
                                                             : GSPH_OK;
        if (st) {
            // this and the later batches' admissions go back to the head of
            // the queue, in their order
            std::vector<Request> back;
            for (size_t q = b; q < plan.size(); ++q)
                for (Request &r : plan[q].admitted) back.push_back(std::move(r));
            std::lock_guard<std::mutex> lock(s->mu);
            for (auto it = back.rbegin(); it != back.rend(); ++it)
                s->queue.push_front(std::move(*it));
            return st;
        }
        std::lock_guard<std::mutex> lock(s->mu);
        std::vector<Request> next;
        next.reserve(pl.keep.size() + pl.admitted.size());
        for (uint32_t k : pl.keep) next.push_back(std::move(sh.resident[k]));
        for (Request &r : pl.admitted) {
            r.pos.clear();
            r.pos.shrink_to_fit();
            r.vel.clear();
            r.vel.shrink_to_fit();
            next.push_back(std::move(r));
        }
        sh.resident = std::move(next);
    }
    // 2. step all resident scenes up to the earliest completion: every batch
    //    is launched on its own stream first, then all are waited for
    uint32_t k = uint32_t(cfg.chunk_frames);
    uint64_t resident_n = 0;
    bool any = false;
    for (const Shard &sh : s->shards)
        for (const Request &r : sh.resident) {
            k = std::min(k, r.remaining);
            resident_n += r.n;
            any = true;
        }
    if (!any) return GSPH_OK;
    gsph_status st = GSPH_OK;
    for (Shard &sh : s->shards)
        if (!sh.resident.empty() && (st = gsph_step(sh.batch, int(k)))) return st;
    for (Shard &sh : s->shards)
        if (!sh.resident.empty() && (st = gsph_sync(sh.batch))) return st;
    // 3. read back the finished requests' final state
    {
        std::lock_guard<std::mutex> lock(s->mu);
        for (Shard &sh : s->shards)
            for (Request &r : sh.resident) r.remaining -= k;
    }
    std::vector<Request> done;
    for (Shard &sh : s->shards) {   // resident lists change only on this thread
        for (size_t i = 0; i < sh.resident.size(); ++i) {
            const Request &r = sh.resident[i];
            if (r.remaining) continue;
            Request out;
            out.id = r.id;
            out.params = r.params;
            out.n = r.n;
            out.frames = r.frames;
            out.pos.resize(size_t(r.n) * 4);
            out.vel.resize(size_t(r.n) * 4);
            if (r.n) {
                if ((st = gsph_copy_out_scene(sh.batch, uint32_t(i), GSPH_FIELD_POSITION,
                                              out.pos.data(), out.pos.size() * 4)) ||
                    (st = gsph_copy_out_scene(sh.batch, uint32_t(i), GSPH_FIELD_VELOCITY,
                                              out.vel.data(), out.vel.size() * 4)))
                    return st;
            }
            done.push_back(std::move(out));
        }
    }
    std::lock_guard<std::mutex> lock(s->mu);
    for (Request &r : done) {
        s->finished_order.push_back(r.id);
        s->finished[r.id] = std::move(r);
        ++s->stats.finished;
    }
    s->stats.frames += k;
    s->stats.chunks += 1;
    s->stats.particle_steps += resident_n * k;
    if (frames_stepped) *frames_stepped = int(k);
    return GSPH_OK;
}

gsph_status gsph_server_poll(gsph_server_handle s, uint64_t *id, uint32_t *n) {
    if (!s || !id) {
        fail("gsph_server_poll: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    while (!s->finished_order.empty() && !s->finished.count(s->finished_order.front()))
        s->finished_order.pop_front();
    if (s->finished_order.empty()) {
        fail("gsph_server_poll: no finished request");
        return GSPH_ERR_STATE;
    }
    *id = s->finished_order.front();
    if (n) *n = s->finished[*id].n;
    return GSPH_OK;
}

gsph_status gsph_server_take(gsph_server_handle s, uint64_t id, float *pos4, float *vel4) {
    if (!s) {
        fail("gsph_server_take: null server");
        return GSPH_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->finished.find(id);
    if (it == s->finished.end()) {
        fail("gsph_server_take: request not finished or already taken");
        return GSPH_ERR_STATE;
    }
    if (pos4 && !it->second.pos.empty())
        std::memcpy(pos4, it->second.pos.data(), it->second.pos.size() * sizeof(float));
    if (vel4 && !it->second.vel.empty())
        std::memcpy(vel4, it->second.vel.data(), it->second.vel.size() * sizeof(float));
    s->finished.erase(it);
    return GSPH_OK;
}

gsph_status gsph_server_get_stats(gsph_server_handle s, gsph_server_stats *out) {
    if (!s || !out) {
        fail("gsph_server_get_stats: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    *out = s->stats;
    out->queued = s->queue.size();
    uint64_t n = 0, bytes = 0, scenes = 0, batches = 0;
    for (const Shard &sh : s->shards) {
        scenes += sh.resident.size();
        batches += sh.resident.empty() ? 0 : 1;
        for (const Request &r : sh.resident) {
            n += r.n;
            bytes += r.bytes();
        }
    }
    out->resident = scenes;
    out->resident_particles = n;
    out->resident_bytes = bytes;
    out->batches = batches;
    return GSPH_OK;
}

}  // extern "C"
