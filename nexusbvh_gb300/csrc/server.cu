// server.cu - a build server: continuous batching under a memory budget.
//
// The reference is a library call per mesh (NXB::BuildBVH8,
// NexusBVH/src/BVHBuilder.cpp:173-267) with no notion of a request stream.
// Here one worker thread owns the GPU side of a server:
//   * requests wait in a FIFO; the worker starts work whenever a stream
//     slot is idle and the request's memory (input copy, scratch, result)
//     fits the budget, letting smaller requests overtake one that does not
//     fit yet;
//   * small 30-bit requests of one prim type that are waiting together are
//     built as one batch (batch.cu: one launch per stage for all of them);
//     the others run the plain allocation-free pipeline (nxb_build_async);
//   * memory comes from a server-owned stream-ordered pool whose release
//     threshold is the budget, so steady-state requests reuse pool memory;
//     scratch is freed in stream order right after each build, results on
//     release;
//   * completion is signalled by a host function enqueued after the build,
//     which only flips an atomic flag and wakes the worker; the worker then
//     reads the per-build error word and counts from pinned memory.
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

#include "pipeline.h"

namespace nxb {
namespace {

using Clock = std::chrono::steady_clock;
constexpr size_t kAlign = 256;
size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct Request {
    uint64_t ticket = 0;
    const void* prims = nullptr;
    bool on_device = false;
    nxb_prim_type type = NXB_PRIM_TRIANGLE;
    uint32_t n = 0;
    nxb_build_config cfg{};
    size_t scratch_bytes = 0;  // input copy + workspace + BVH2, freed after the build
    size_t result_bytes = 0;   // BVH8 nodes + primIdx, freed on release
    Clock::time_point t_submit, t_start, t_done;
    double dev_start_ms = 0.0, dev_end_ms = 0.0;  // since the server's base event
    unsigned char* result = nullptr;
    nxb_bvh8 bvh8{};
    nxb_status status = NXB_OK;
    uint32_t batched_with = 1;
    bool done = false;
};

size_t prim_bytes(nxb_prim_type t) { return t == NXB_PRIM_TRIANGLE ? 36 : 24; }

struct Slot;

struct Job {
    std::vector<Request*> reqs;
    bool batched = false;
    size_t scratch_bytes = 0;
    unsigned char* scratch = nullptr;  // until its stream-ordered free is enqueued
    std::atomic<bool> complete{false};
    Clock::time_point t_done;
    Slot* slot = nullptr;
    std::condition_variable* wake = nullptr;
};

// Pinned per-slot staging: a slot runs one job at a time.
struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_end = nullptr;  // the running job's device interval
    Job* job = nullptr;
    nxb_build_result* h_result = nullptr;  // plain builds
    uint32_t* h_err = nullptr;             // batched builds
    uint32_t* h_off = nullptr;             // batch_max_meshes + 1
    uint32_t* h_off8 = nullptr;            // batch_max_meshes + 1
    nxb_batch_mesh* h_meshes = nullptr;    // batch_max_meshes
};

}  // namespace
}  // namespace nxb

using namespace nxb;

struct nxb_server {
    nxb_server_config cfg{};
    int device = 0;
    cudaEvent_t base = nullptr;  // device time zero of the request intervals
    cudaMemPool_t pool = nullptr;
    cudaStream_t release_stream = nullptr;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work;  // worker wake-up
    std::condition_variable cv_done;  // waiters
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> all;
    uint64_t next_ticket = 1;
    size_t in_use = 0;
    nxb_server_stats stats{};
    bool stop = false;
    std::thread worker;
};

namespace {

// Host function enqueued after a build: no CUDA calls, no lock.
void CUDART_CB on_job_done(void* p) {
    Job* j = static_cast<Job*>(p);
    j->t_done = Clock::now();
    std::condition_variable* wake = j->wake;
    j->complete.store(true, std::memory_order_release);
    wake->notify_one();
}

nxb_status status_of_word(uint32_t w) {
    if (w == 0) return NXB_OK;
    if (w & (NXB_DEVERR_SORT_LOOKBACK_TIMEOUT | NXB_DEVERR_BVH8_QUEUE_TIMEOUT)) return NXB_ERR_DEVICE_TIMEOUT;
    return NXB_ERR_DEVICE_INVARIANT;
}

bool batchable(const nxb_server* s, const Request* r) {
    return r->n <= s->cfg.batch_max_prims && r->cfg.prioritize_speed && s->cfg.batch_max_prims > 1;
}

// Memory of a plain build: input copy, workspace, BVH2 (scratch); BVH8 and
// primIdx (result).
void size_plain(Request* r) {
    nxb_build_sizes sz{};
    nxb_query_build_sizes(r->n, &r->cfg, &sz);
    r->scratch_bytes = (r->on_device ? 0 : align_up(prim_bytes(r->type) * r->n)) + align_up(sz.workspace_bytes) +
                       align_up(sizeof(nxb_bvh2_node) * sz.bvh2_node_count) + kAlign;
    r->result_bytes = align_up(sizeof(nxb_bvh8_node) * sz.bvh8_node_capacity) + align_up(4ull * r->n);
}

cudaError_t alloc(nxb_server* s, void** p, size_t bytes, cudaStream_t st) {
    return cudaMallocFromPoolAsync(p, bytes ? bytes : kAlign, s->pool, st);
}

// Launches a job on its slot; on failure marks its requests failed.
nxb_status launch_plain(nxb_server* s, Job* j) {
    Request* r = j->reqs[0];
    Slot* sl = j->slot;
    cudaStream_t st = sl->stream;
    nxb_build_sizes sz{};
    nxb_query_build_sizes(r->n, &r->cfg, &sz);
    unsigned char* scratch = nullptr;
    cudaError_t e = alloc(s, (void**)&scratch, r->scratch_bytes, st);
    if (e) return record_cuda_error(e);
    j->scratch = scratch;
    e = alloc(s, (void**)&r->result, r->result_bytes, st);
    if (e) return record_cuda_error(e);
    size_t at = 0;
    const void* prims = r->prims;
    e = cudaEventRecord(sl->ev_start, st);
    if (e) return record_cuda_error(e);
    if (!r->on_device) {
        prims = scratch;
        e = cudaMemcpyAsync(scratch, r->prims, prim_bytes(r->type) * r->n, cudaMemcpyHostToDevice, st);
        at += align_up(prim_bytes(r->type) * r->n);
    }
    unsigned char* ws = scratch + at;
    at += align_up(sz.workspace_bytes);
    nxb_bvh2_node* b2 = reinterpret_cast<nxb_bvh2_node*>(scratch + at);
    at += align_up(sizeof(nxb_bvh2_node) * sz.bvh2_node_count);
    nxb_build_result* d_res = reinterpret_cast<nxb_build_result*>(scratch + at);
    nxb_bvh8_node* b8 = reinterpret_cast<nxb_bvh8_node*>(r->result);
    uint32_t* prim = reinterpret_cast<uint32_t*>(r->result + align_up(sizeof(nxb_bvh8_node) * sz.bvh8_node_capacity));
    if (e) return record_cuda_error(e);
    nxb_status stt = nxb_build_async(prims, r->type, r->n, &r->cfg, ws, sz.workspace_bytes, b2, b8, prim, d_res, st);
    if (stt != NXB_OK) return stt;
    e = cudaMemcpyAsync(sl->h_result, d_res, sizeof(nxb_build_result), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaEventRecord(sl->ev_end, st);
    if (!e) e = cudaFreeAsync(scratch, st);
    if (!e) j->scratch = nullptr;
    if (!e) e = cudaLaunchHostFunc(st, on_job_done, j);
    r->bvh8.nodes = b8;
    r->bvh8.prim_idx = prim;
    r->bvh8.prim_count = r->n;
    return e ? record_cuda_error(e) : NXB_OK;
}

nxb_status launch_batch(nxb_server* s, Job* j) {
    Slot* sl = j->slot;
    cudaStream_t st = sl->stream;
    const uint32_t M = (uint32_t)j->reqs.size();
    const nxb_prim_type type = j->reqs[0]->type;
    sl->h_off[0] = 0;
    for (uint32_t m = 0; m < M; ++m) sl->h_off[m + 1] = sl->h_off[m] + j->reqs[m]->n;
    BatchArena a;
    if (!batch_layout(sl->h_off, M, sl->h_off8, &a)) return NXB_ERR_UNSUPPORTED;
    const size_t in_bytes = align_up(prim_bytes(type) * (size_t)a.total);
    unsigned char* scratch = nullptr;
    cudaError_t e = alloc(s, (void**)&scratch, in_bytes + a.bytes, st);
    if (e) return record_cuda_error(e);
    j->scratch = scratch;
    for (uint32_t m = 0; m < M && !e; ++m) e = alloc(s, (void**)&j->reqs[m]->result, j->reqs[m]->result_bytes, st);
    if (e) return record_cuda_error(e);
    batch_bind(scratch + in_bytes, &a);
    e = cudaEventRecord(sl->ev_start, st);
    // the meshes end to end
    for (uint32_t m = 0; m < M && !e; ++m) {
        const Request* r = j->reqs[m];
        e = cudaMemcpyAsync(scratch + prim_bytes(type) * sl->h_off[m], r->prims, prim_bytes(type) * r->n,
                            r->on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st);
    }
    if (!e) e = cudaMemcpyAsync(a.off, sl->h_off, 4ull * (M + 1), cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(a.off8, sl->h_off8, 4ull * (M + 1), cudaMemcpyHostToDevice, st);
    if (e) return record_cuda_error(e);
    BatchTuning t;
    t.radius = j->reqs[0]->cfg.search_radius ? j->reqs[0]->cfg.search_radius : 8u;
    t.auction = (j->reqs[0]->cfg.flags & NXB_BUILD_AUCTION) != 0;
    nxb_status stt = batch_enqueue(a, scratch, type, t, sl->h_err, st);
    if (stt != NXB_OK) return stt;
    // each mesh's BVH8 into its request's own result memory
    for (uint32_t m = 0; m < M && !e; ++m) {
        Request* r = j->reqs[m];
        const size_t cap = batch_bvh8_capacity(r->n);
        nxb_bvh8_node* b8 = reinterpret_cast<nxb_bvh8_node*>(r->result);
        uint32_t* prim = reinterpret_cast<uint32_t*>(r->result + align_up(sizeof(nxb_bvh8_node) * cap));
        e = cudaMemcpyAsync(b8, a.bvh8 + sl->h_off8[m], sizeof(nxb_bvh8_node) * cap, cudaMemcpyDeviceToDevice, st);
        if (!e)
            e = cudaMemcpyAsync(prim, a.prim_idx + sl->h_off[m], 4ull * r->n, cudaMemcpyDeviceToDevice, st);
        r->bvh8.nodes = b8;
        r->bvh8.prim_idx = prim;
        r->bvh8.prim_count = r->n;
    }
    if (!e) e = cudaMemcpyAsync(sl->h_meshes, a.results, sizeof(nxb_batch_mesh) * M, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaEventRecord(sl->ev_end, st);
    if (!e) e = cudaFreeAsync(scratch, st);
    if (!e) j->scratch = nullptr;
    if (!e) e = cudaLaunchHostFunc(st, on_job_done, j);
    return e ? record_cuda_error(e) : NXB_OK;
}

// Called with the lock held: the completed job's outcome into its requests.
void reap(nxb_server* s, Slot& sl) {
    Job* j = sl.job;
    if (j->batched) {
        const nxb_status st = status_of_word(*sl.h_err);
        for (size_t m = 0; m < j->reqs.size(); ++m) {
            Request* r = j->reqs[m];
            r->status = st;
            r->bvh8.node_count = sl.h_meshes[m].bvh8_node_count;
            r->bvh8.bounds = sl.h_meshes[m].scene_bounds;
        }
    } else {
        Request* r = j->reqs[0];
        r->status = status_of_word(sl.h_result->error_word);
        r->bvh8.node_count = sl.h_result->bvh8_node_count;
        r->bvh8.bounds = sl.h_result->scene_bounds;
    }
    // the job's events have completed (its host function ran after them)
    float t0 = 0.f, t1 = 0.f;
    if (cudaEventElapsedTime(&t0, s->base, sl.ev_start) != cudaSuccess ||
        cudaEventElapsedTime(&t1, s->base, sl.ev_end) != cudaSuccess)
        t0 = t1 = -1.f;
    for (Request* r : j->reqs) {
        r->t_done = j->t_done;
        r->dev_start_ms = t0;
        r->dev_end_ms = t1;
        r->done = true;
        r->batched_with = (uint32_t)j->reqs.size();
        if (r->status != NXB_OK && r->result) {
            cudaFreeAsync(r->result, s->release_stream);
            r->result = nullptr;
            s->in_use -= r->result_bytes;
        }
    }
    s->in_use -= j->scratch_bytes;
    s->stats.completed += j->reqs.size();
    delete j;
    sl.job = nullptr;
}

void fail_job(nxb_server* s, Job* j, nxb_status st) {
    // nothing of the job runs any more; what it allocated is freed once the
    // stream has drained (the worker waits for that before reusing the slot)
    cudaStreamSynchronize(j->slot->stream);
    if (j->scratch) cudaFreeAsync(j->scratch, j->slot->stream);
    for (Request* r : j->reqs) {
        if (r->result) {
            cudaFreeAsync(r->result, j->slot->stream);
            r->result = nullptr;
        }
        s->in_use -= r->result_bytes;
        r->status = st;
        r->done = true;
        r->t_done = Clock::now();
    }
    s->in_use -= j->scratch_bytes;
    s->stats.completed += j->reqs.size();
    delete j;
}

// Picks the next job from the queue (lock held): the first request that
// fits, plus, if it can be batched, every later waiting request that can
// join it (same prim type and radius) and fits.
Job* pick(nxb_server* s) {
    const size_t budget = s->cfg.memory_budget_bytes;
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
        Request* r = *it;
        if (s->in_use + r->scratch_bytes + r->result_bytes > budget) continue;
        Job* j = new Job();
        if (!batchable(s, r)) {
            j->reqs.push_back(r);
            j->scratch_bytes = r->scratch_bytes;
            s->in_use += r->scratch_bytes + r->result_bytes;
            s->queue.erase(it);
            return j;
        }
        j->batched = true;
        size_t total = 0;
        std::vector<Request*> take;
        size_t extra = 0;
        for (auto jt = it; jt != s->queue.end() && take.size() < s->cfg.batch_max_meshes; ++jt) {
            Request* q = *jt;
            if (!batchable(s, q) || q->type != r->type || q->cfg.search_radius != r->cfg.search_radius ||
                q->cfg.flags != r->cfg.flags)
                continue;
            const size_t need = q->scratch_bytes + q->result_bytes;
            if (s->in_use + extra + need > budget) continue;
            if (total + q->n > (1u << 30) - 1) break;
            take.push_back(q);
            extra += need;
            total += q->n;
        }
        for (Request* q : take) {
            for (auto kt = s->queue.begin(); kt != s->queue.end(); ++kt)
                if (*kt == q) {
                    s->queue.erase(kt);
                    break;
                }
            j->reqs.push_back(q);
            j->scratch_bytes += q->scratch_bytes;
        }
        s->in_use += extra;
        return j;
    }
    return nullptr;
}

void worker_main(nxb_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        bool progressed = false;
        for (Slot& sl : s->slots)
            if (sl.job && sl.job->complete.load(std::memory_order_acquire)) {
                reap(s, sl);
                progressed = true;
            }
        if (progressed) s->cv_done.notify_all();
        if (s->stop) {
            bool busy = false;
            for (Slot& sl : s->slots) busy |= sl.job != nullptr;
            if (!busy) break;
        }
        for (Slot& sl : s->slots) {
            if (sl.job || s->stop) continue;
            Job* j = pick(s);
            if (!j) break;
            j->slot = &sl;
            j->wake = &s->cv_work;
            const Clock::time_point now = Clock::now();
            for (Request* r : j->reqs) r->t_start = now;
            s->stats.builds++;
            if (j->reqs.size() > 1) {
                s->stats.batched_builds++;
                s->stats.batched_requests += j->reqs.size();
            }
            if (s->in_use > s->stats.peak_bytes_in_use) s->stats.peak_bytes_in_use = s->in_use;
            const nxb_status st = j->batched ? launch_batch(s, j) : launch_plain(s, j);
            if (st != NXB_OK) {
                fail_job(s, j, st);
                s->cv_done.notify_all();
                continue;
            }
            sl.job = j;
            progressed = true;
        }
        if (!progressed) s->cv_work.wait_for(lk, std::chrono::microseconds(200));
    }
    lk.unlock();
    for (Slot& sl : s->slots) cudaStreamSynchronize(sl.stream);
}

void destroy_server(nxb_server* s) {
    for (auto& kv : s->all)
        if (kv.second->result) cudaFreeAsync(kv.second->result, s->release_stream);
    if (s->release_stream) cudaStreamSynchronize(s->release_stream);
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.ev_start) cudaEventDestroy(sl.ev_start);
        if (sl.ev_end) cudaEventDestroy(sl.ev_end);
        if (sl.h_result) cudaFreeHost(sl.h_result);
        if (sl.h_err) cudaFreeHost(sl.h_err);
        if (sl.h_off) cudaFreeHost(sl.h_off);
        if (sl.h_off8) cudaFreeHost(sl.h_off8);
        if (sl.h_meshes) cudaFreeHost(sl.h_meshes);
    }
    if (s->release_stream) cudaStreamDestroy(s->release_stream);
    if (s->base) cudaEventDestroy(s->base);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
}

void fill_result(const Request* r, nxb_server_result* out) {
    out->bvh8 = r->bvh8;
    out->status = (int32_t)r->status;
    out->batched_with = r->batched_with;
    out->queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
    out->latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    out->device_start_ms = r->dev_start_ms;
    out->device_end_ms = r->dev_end_ms;
}

// One tiny build through each pipeline a server runs at the default radius:
// plain 30-bit and 63-bit, and batched, for triangles and boxes.  The CUDA
// runtime loads a kernel on its first launch (lazy module loading); without
// this, the first batched build of a server's life stalls the worker thread
// for tens of milliseconds while every request behind it waits.
nxb_status warm_up(cudaStream_t st) {
    constexpr uint32_t kTris = 96, kMeshes = 2;
    std::vector<float> h(9 * kTris);
    for (uint32_t k = 0; k < kTris; ++k) {
        const float x = (float)(k % 7), y = (float)(k / 7 % 5), z = (float)(k / 35);
        const float v[9] = {x, y, z, x + 0.5f, y, z + 0.25f, x, y + 0.5f, z + 0.5f};
        std::memcpy(&h[9 * k], v, sizeof v);
    }
    std::vector<float> hb(6 * kTris);  // the triangles' boxes
    for (uint32_t k = 0; k < kTris; ++k)
        for (int a = 0; a < 3; ++a) {
            const float* t = &h[9 * k];
            hb[6 * k + a] = std::min(t[a], std::min(t[3 + a], t[6 + a]));
            hb[6 * k + 3 + a] = std::max(t[a], std::max(t[3 + a], t[6 + a]));
        }
    void* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(float) * (h.size() + hb.size()));
    if (e) return record_cuda_error(e);
    float* d_tri = static_cast<float*>(d);
    float* d_box = d_tri + h.size();
    e = cudaMemcpy(d_tri, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d_box, hb.data(), sizeof(float) * hb.size(), cudaMemcpyHostToDevice);
    nxb_status st_out = e ? record_cuda_error(e) : NXB_OK;
    const uint32_t off[kMeshes + 1] = {0, kTris / 2, kTris};
    for (int type = 0; type < 2 && st_out == NXB_OK; ++type) {
        const nxb_prim_type pt = type ? NXB_PRIM_TRIANGLE : NXB_PRIM_AABB;
        const void* prims = type ? (const void*)d_tri : (const void*)d_box;
        for (uint32_t fast = 0; fast < 2 && st_out == NXB_OK; ++fast) {
            nxb_build_config cfg{};
            cfg.prioritize_speed = fast;
            nxb_bvh8 out{};
            st_out = nxb_build_bvh8(prims, pt, kTris, &cfg, st, &out, nullptr);
            if (st_out == NXB_OK) nxb_free_device_bvh8(&out);
        }
        if (st_out == NXB_OK) {
            nxb_build_config cfg{};
            cfg.prioritize_speed = 1;
            nxb_batch* b = nullptr;
            st_out = nxb_batch_create(pt, off, kMeshes, &cfg, &b);
            if (st_out == NXB_OK) {
                st_out = nxb_batch_build(b, prims, st, nullptr);
                nxb_batch_destroy(b);
            }
        }
    }
    cudaFree(d);
    return st_out;
}

}  // namespace

extern "C" {

nxb_status nxb_server_create(const nxb_server_config* config, nxb_server** out) {
    if (!out) return NXB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    nxb_server_config c = config ? *config : nxb_server_config{};
    if (c.flags & ~NXB_SERVER_RESERVE) return NXB_ERR_UNSUPPORTED;
    if (c.memory_budget_bytes == 0) c.memory_budget_bytes = 32ull << 30;
    if (c.streams == 0) c.streams = 4;
    if (c.streams > 64) return NXB_ERR_UNSUPPORTED;
    if (c.batch_max_prims == 0) c.batch_max_prims = 65536;
    if (c.batch_max_meshes == 0) c.batch_max_meshes = 256;
    if (c.batch_max_meshes > 65536) return NXB_ERR_UNSUPPORTED;
    nxb_server* s = new nxb_server();
    s->cfg = c;
    cudaError_t e = cudaGetDevice(&s->device);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    if (!e) e = cudaMemPoolCreate(&s->pool, &props);
    if (!e) {
        uint64_t keep = c.memory_budget_bytes;
        e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (!e) e = cudaStreamCreateWithFlags(&s->release_stream, cudaStreamNonBlocking);
    s->slots.resize(c.streams);
    for (Slot& sl : s->slots) {
        if (!e) e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (!e) e = cudaEventCreate(&sl.ev_start);
        if (!e) e = cudaEventCreate(&sl.ev_end);
        if (!e) e = cudaMallocHost(&sl.h_result, sizeof(nxb_build_result));
        if (!e) e = cudaMallocHost(&sl.h_err, sizeof(uint32_t));
        if (!e) e = cudaMallocHost(&sl.h_off, 4ull * (c.batch_max_meshes + 1));
        if (!e) e = cudaMallocHost(&sl.h_off8, 4ull * (c.batch_max_meshes + 1));
        if (!e) e = cudaMallocHost(&sl.h_meshes, sizeof(nxb_batch_mesh) * c.batch_max_meshes);
    }
    if (!e && (c.flags & NXB_SERVER_RESERVE)) {
        // take the whole budget into the pool once (it keeps up to the
        // budget when freed), so that no request waits on the pool growing
        void* p = nullptr;
        e = cudaMallocFromPoolAsync(&p, c.memory_budget_bytes, s->pool, s->release_stream);
        if (!e) e = cudaFreeAsync(p, s->release_stream);
        if (!e) e = cudaStreamSynchronize(s->release_stream);
    }
    if (e) {
        const nxb_status st = record_cuda_error(e);
        destroy_server(s);
        return st;
    }
    const nxb_status wst = warm_up(s->slots[0].stream);
    if (wst != NXB_OK) {
        destroy_server(s);
        return wst;
    }
    e = cudaEventCreate(&s->base);
    if (!e) e = cudaEventRecord(s->base, s->release_stream);
    if (!e) e = cudaEventSynchronize(s->base);
    if (e) {
        const nxb_status st = record_cuda_error(e);
        destroy_server(s);
        return st;
    }
    s->worker = std::thread(worker_main, s);
    *out = s;
    return NXB_OK;
}

nxb_status nxb_server_destroy(nxb_server* s) {
    if (!s) return NXB_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        // queued requests that never started complete as failed
        for (Request* r : s->queue) {
            r->status = NXB_ERR_INVALID_ARGUMENT;
            r->done = true;
        }
        s->queue.clear();
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    s->cv_done.notify_all();
    destroy_server(s);
    return NXB_OK;
}

nxb_status nxb_server_submit(nxb_server* s, const void* prims, int on_device, nxb_prim_type type, uint32_t n,
                             const nxb_build_config* cfg, uint64_t* ticket) {
    if (!s || !prims || !ticket || n == 0) return NXB_ERR_INVALID_ARGUMENT;
    if (type != NXB_PRIM_AABB && type != NXB_PRIM_TRIANGLE) return NXB_ERR_INVALID_ARGUMENT;
    if (n > (1u << 30) - 1) return NXB_ERR_UNSUPPORTED;
    if (cfg) {
        const uint32_t r = cfg->search_radius;
        if ((r != 0 && r != 4 && r != 8 && r != 16) || (cfg->flags & ~NXB_BUILD_AUCTION)) return NXB_ERR_UNSUPPORTED;
    }
    auto req = std::make_unique<Request>();
    req->prims = prims;
    req->on_device = on_device != 0;
    req->type = type;
    req->n = n;
    if (cfg) req->cfg = *cfg;
    if (req->cfg.search_radius == 0) req->cfg.search_radius = 8;
    if (batchable(s, req.get())) {
        // a share of a batched build: input copy, arena, result
        BatchArena a;
        uint32_t off[2] = {0, n}, off8[2];
        batch_layout(off, 1, off8, &a);
        req->scratch_bytes = align_up(prim_bytes(type) * (size_t)n) + a.bytes;
        req->result_bytes = align_up(sizeof(nxb_bvh8_node) * (size_t)batch_bvh8_capacity(n)) + align_up(4ull * n);
    } else {
        size_plain(req.get());
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (req->scratch_bytes + req->result_bytes > s->cfg.memory_budget_bytes) {
        s->stats.rejected++;
        return NXB_ERR_ADMISSION;
    }
    req->ticket = s->next_ticket++;
    req->t_submit = Clock::now();
    *ticket = req->ticket;
    s->queue.push_back(req.get());
    s->all.emplace(req->ticket, std::move(req));
    s->stats.submitted++;
    s->cv_work.notify_one();
    return NXB_OK;
}

nxb_status nxb_server_wait(nxb_server* s, uint64_t ticket, nxb_server_result* out) {
    if (!s) return NXB_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return NXB_ERR_INVALID_ARGUMENT;
    Request* r = it->second.get();
    s->cv_work.notify_one();
    while (!r->done) s->cv_done.wait_for(lk, std::chrono::milliseconds(1));
    if (out) fill_result(r, out);
    return r->status;
}

nxb_status nxb_server_poll(nxb_server* s, uint64_t ticket, nxb_server_result* out, int* done) {
    if (!s || !done) return NXB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return NXB_ERR_INVALID_ARGUMENT;
    Request* r = it->second.get();
    *done = r->done ? 1 : 0;
    if (r->done && out) fill_result(r, out);
    return NXB_OK;
}

nxb_status nxb_server_release(nxb_server* s, uint64_t ticket) {
    if (!s) return NXB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end() || !it->second->done) return NXB_ERR_INVALID_ARGUMENT;
    Request* r = it->second.get();
    if (r->result) {
        const cudaError_t e = cudaFreeAsync(r->result, s->release_stream);
        s->in_use -= r->result_bytes;
        s->all.erase(it);
        s->cv_work.notify_one();
        return e ? record_cuda_error(e) : NXB_OK;
    }
    s->all.erase(it);
    return NXB_OK;
}

nxb_status nxb_server_get_stats(nxb_server* s, nxb_server_stats* out) {
    if (!s || !out) return NXB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->bytes_in_use = s->in_use;
    return NXB_OK;
}

}  // extern "C"
