/*
 * server.cu -- a request server over device-resident trees: frame and
 * ball-collision requests from any number of client threads, admitted by a
 * device-memory budget and batched continuously onto the GPU.
 *
 * Continuous batching.  A worker thread repeats: retire finished launches
 * (returning their memory to the budget), admit waiting requests in arrival
 * order while the budget and the in-flight slots allow, and put everything
 * admitted since the previous launch into one launch on the next of several
 * streams -- all frames into one persistent work-queue kernel (the batched
 * kernel of batch.cu), each ball request into the ball kernel.  Frames are
 * drawn into device memory and copied into the pinned host buffers the
 * clients read as soon as their launch's kernel ends (frame stores straight
 * into host memory slow the frame kernel by a third).  A frame is zero
 * outside its tree's screen rectangle, and a reused buffer is zero outside
 * the rectangle of the frame it held last, so only the box covering both
 * crosses to the host (about a sixth of the bytes on a mixed load).  Ball
 * hits, one byte a query, are written in place by the ball kernel, which
 * also reads its staged inputs from pinned memory.  The device budget holds the resident trees,
 * the per-launch job tables and the frames being drawn; the pinned-host
 * budget holds the results and staged inputs.
 * Requests that arrive while earlier launches are still on the GPU go out
 * in the next launch and overlap with them on the device instead of waiting
 * for them.
 *
 * Every result is the one the plain entry points give for the same request
 * alone (vox_cuda_render_device, vox_cuda_ball_batch): same kernels, same
 * trees, no state shared between requests.
 *
 * Waiting is bounded: vox_cuda_server_wait gives up after its timeout with
 * VOX_CUDA_ETIMEOUT; a request that can never fit the budget is refused at
 * submission with VOX_CUDA_EBUDGET.
 */
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
#include <unordered_map>
#include <vector>

#include "internal.h"
#include "abi_guard.h"

#define EXPORT extern "C" __attribute__((visibility("default")))

namespace {

uint64_t now_ns()
{
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Size class of a pinned buffer: the next power of two from 4 KiB.
size_t pinned_class(size_t bytes)
{
    size_t cls = 4096;
    while (cls < bytes) cls <<= 1;
    return cls;
}

// What a pinned buffer may still hold from its last use.  Every byte below
// `tail` that lies outside rectangle [x0, x1) x [y0, y1) of a frame w pixels
// wide (row pitch w * 4 bytes) is zero; bytes from `tail` on may hold
// anything.  A buffer of unknown contents -- new, or last used for ball
// results or by a request that failed -- has w = 0 and tail = 0.
struct Dirty {
    uint32_t w = 0, x0 = 0, y0 = 0, x1 = 0, y1 = 0;
    size_t tail = 0;
};

// The part of a w x h frame to copy into a buffer whose state is `d`, given
// that the device frame is zero outside rectangle r ({x0, y0, x1, y1} of
// frame_rect_of: no pixel outside it sees the tree).  Either the whole frame
// (`full`), or the box [x0, x1) x [y0, y1), which covers the frame's
// rectangle and what the buffer's last frame left non-zero (same row pitch),
// or nothing (both empty).  `after` is the buffer's state once it is copied.
struct FrameCopy {
    bool full = false;
    uint32_t x0 = 0, y0 = 0, x1 = 0, y1 = 0;
};

FrameCopy plan_frame_copy(const Dirty &d, uint32_t w, uint32_t h, const uint32_t r[4], Dirty &after)
{
    const size_t fb = (size_t)w * h * 4;
    const uint32_t rx1 = std::min(r[2], w), ry1 = std::min(r[3], h);
    const bool have = rx1 > r[0] && ry1 > r[1];
    const bool had = d.w != 0 && d.x1 > d.x0 && d.y1 > d.y0;
    FrameCopy c;
    if (d.w == w && d.tail >= fb) {
        // below fb the buffer is zero outside d's rectangle, in this pitch
        const uint32_t oy1 = std::min(d.y1, h);
        const bool old_in = had && oy1 > d.y0;
        if (have || old_in) {
            c.x0 = have ? r[0] : d.x0;
            c.y0 = have ? r[1] : d.y0;
            c.x1 = have ? rx1 : d.x1;
            c.y1 = have ? ry1 : oy1;
            if (have && old_in) {
                c.x0 = std::min(c.x0, d.x0);
                c.y0 = std::min(c.y0, d.y0);
                c.x1 = std::max(c.x1, d.x1);
                c.y1 = std::max(c.y1, oy1);
            }
        }
        // rows of the old rectangle below the frame lie past fb
        after.tail = (had && d.y1 > h) ? fb : d.tail;
    } else {
        c.full = true;
        const size_t old_end = had ? (size_t)d.y1 * d.w * 4 : 0;
        after.tail = (d.tail <= fb || old_end > fb) ? fb : d.tail;
    }
    after.w = w;
    after.x0 = have ? r[0] : 0;
    after.y0 = have ? r[1] : 0;
    after.x1 = have ? rx1 : 0;
    after.y1 = have ? ry1 : 0;
    return c;
}

// Pinned host buffers by power-of-two size class, reused across requests.
// Buffers up to 64 MiB are carved from 128 MiB pinned slabs; a part of the
// host budget is pinned in slabs when the server starts, and a refill thread
// keeps two slabs pinned ahead of the one being carved, so the worker thread
// -- which admits and launches every request -- does not stop for
// page-locking (14 GB/s on the Grace host: 4.5 ms for one 64 MiB buffer).
// With no slab room ready, a free buffer of a larger class serves before the
// worker pins one itself.  Larger buffers are pinned one by one.  Buffers go
// back to their class's free list with their Dirty state, and slabs stay
// pinned until the pool is destroyed.
class PinnedPool {
  public:
    static constexpr size_t SLAB = size_t(128) << 20, MAX_CARVED = size_t(64) << 20, SPARES = 2;

    ~PinnedPool()
    {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        if (refill_.joinable()) refill_.join();
        for (void *p : slabs_) cudaFreeHost(p);
        for (void *p : spares_) cudaFreeHost(p);
        for (void *p : direct_) cudaFreeHost(p);
    }

    // Pins `now` bytes (whole slabs) at once and starts the refill thread for
    // device `dev`, which pins further slabs while fewer than `cap` bytes are
    // in slabs.  Returns false if the first slabs cannot be pinned.
    bool start(int dev, size_t now, size_t cap)
    {
        dev_ = dev;
        cap_ = cap;
        for (size_t got = 0; got + SLAB <= now; got += SLAB) {
            void *p = nullptr;
            if (cudaHostAlloc(&p, SLAB, cudaHostAllocDefault) != cudaSuccess) return false;
            spares_.push_back(p);
            pinned_ += SLAB;
        }
        refill_ = std::thread([this] { refill_loop(); });
        return true;
    }

    // A buffer of at least `bytes`; *dirty (may be NULL) gets what it holds.
    void *get(size_t bytes, size_t *cls_out, Dirty *dirty = nullptr)
    {
        size_t cls = pinned_class(bytes);
        *cls_out = cls;
        if (dirty) *dirty = Dirty{};
        {
            std::lock_guard<std::mutex> lk(mu_);
            auto &v = free_[cls];
            if (!v.empty()) {
                void *p = v.back().first;
                if (dirty) *dirty = v.back().second;
                v.pop_back();
                return p;
            }
            if (cls <= MAX_CARVED) {
                if (cur_used_ + cls > SLAB && !spares_.empty()) {   // next slab, pinned ahead
                    cur_ = static_cast<char *>(spares_.back());
                    spares_.pop_back();
                    slabs_.push_back(cur_);
                    cur_used_ = 0;
                    cv_.notify_all();
                }
                if (cur_ && cur_used_ + cls <= SLAB) {
                    void *p = cur_ + cur_used_;
                    cur_used_ += cls;
                    return p;
                }
            }
            // no slab room ready: a free buffer of a class up to 8x larger
            // serves before anything is pinned here
            for (size_t big = cls << 1; big <= cls << 3; big <<= 1) {
                auto it = free_.find(big);
                if (it == free_.end() || it->second.empty()) continue;
                void *p = it->second.back().first;
                if (dirty) *dirty = it->second.back().second;
                it->second.pop_back();
                *cls_out = big;
                return p;
            }
        }
        // no slab room ready (or a buffer larger than a slab carves): pin here
        void *p = nullptr;
        uint64_t t0 = now_ns();
        cudaError_t e = cudaMallocHost(&p, cls);
        pin_ns.fetch_add(now_ns() - t0, std::memory_order_relaxed);
        pins.fetch_add(1, std::memory_order_relaxed);
        if (e != cudaSuccess) return nullptr;
        std::lock_guard<std::mutex> lk(mu_);
        direct_.push_back(p);
        return p;
    }
    std::atomic<uint64_t> pin_ns{0}, pins{0};   // time and count of buffers the worker pinned itself
    uint64_t slabs()
    {
        std::lock_guard<std::mutex> lk(mu_);
        return pinned_ / SLAB;
    }
    void put(void *p, size_t cls, const Dirty &dirty = Dirty{})
    {
        if (!p) return;
        std::lock_guard<std::mutex> lk(mu_);
        free_[cls].push_back({p, dirty});
    }

  private:
    // Keeps SPARES slabs pinned ahead while the pool lives.
    void refill_loop()
    {
        cudaSetDevice(dev_);
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_.wait(lk, [this] { return stop_ || (spares_.size() < SPARES && pinned_ + SLAB <= cap_); });
            if (stop_) return;
            lk.unlock();
            void *p = nullptr;
            bool ok = cudaHostAlloc(&p, SLAB, cudaHostAllocDefault) == cudaSuccess;
            lk.lock();
            if (!ok) return;        // out of pinnable memory: the worker pins what it needs itself
            spares_.push_back(p);
            pinned_ += SLAB;
        }
    }

    std::mutex mu_;
    std::condition_variable cv_;
    std::map<size_t, std::vector<std::pair<void *, Dirty>>> free_;
    std::vector<void *> slabs_, spares_, direct_;
    char *cur_ = nullptr;
    size_t cur_used_ = SLAB;
    size_t pinned_ = 0, cap_ = 0;   // bytes in slabs, and the most the refill thread pins
    int dev_ = 0;
    bool stop_ = false;
    std::thread refill_;
};

enum Kind { FRAME = 0, BALLS = 1 };

struct Request {
    uint64_t ticket = 0;
    Kind kind = FRAME;
    uint32_t tree = 0;
    vox_cuda_camera cam{};
    uint32_t w = 0, h = 0, n = 0;
    std::vector<float> centres, radii;
    uint64_t dev_bytes = 0;         // charged to the device budget while admitted
    uint64_t host_bytes = 0;        // charged to the pinned-host budget while admitted
    void *h_res = nullptr;          // pinned result, written in place by the kernels
    size_t h_cls = 0, res_bytes = 0;
    Dirty h_dirty;                  // what h_res holds: as taken from the pool, then after this frame's copy
    void *d_res = nullptr;          // a frame kept in device memory (frames_on_device)
    uint64_t dev_hold = 0;          // device bytes still charged after the launch ends (until release)
    void *h_in = nullptr;           // pinned ball inputs
    size_t h_in_cls = 0;
    uint64_t t_submit = 0, t_launch = 0, t_done = 0;
    int status = VOX_CUDA_OK;
    bool done = false;
};

struct Launch {
    vox_cuda_server *srv = nullptr;
    std::vector<Request *> reqs;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;     // recorded after the result copies
    void *h_table = nullptr;
    size_t h_table_cls = 0;
    void *d_table = nullptr;        // job table + queue head
    void *d_frames = nullptr;       // the launch's frames, drawn here before their copies
    std::atomic<bool> finished{false};   // set by the stream callback
    std::atomic<uint64_t> t_cb{0};       // completion time seen by the callback
    bool has_callback = false;      // then only `finished` may retire the launch
    // buffers to give back once retired (taken off the requests under the lock)
    std::vector<std::pair<void *, size_t>> host_free;
};

}  // namespace

struct vox_cuda_server {
    vox_cuda_server_config cfg{};
    int device = 0, nsm = 0;
    std::vector<const vox_cuda_tree *> trees;
    uint8_t *d_tex = nullptr;
    std::vector<cudaStream_t> streams;
    size_t next_stream = 0;
    PinnedPool pinned;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> pending;
    std::vector<Request *> admitted;
    std::vector<Launch *> inflight;
    std::unordered_map<uint64_t, Request *> reqs;
    uint64_t next_ticket = 1;
    uint64_t used = 0, peak = 0, tree_bytes = 0, host_used = 0, host_peak = 0;
    uint64_t submitted = 0, completed = 0, rejected = 0, launches = 0;
    uint32_t inflight_reqs = 0;
    uint32_t building = 0;          // launches being built outside the lock
    bool stop = false;
    bool failed = false;            // the worker stopped on a failure: requests are refused
    std::atomic<int> inject{0};     // host-side fault for the next launch (vox_cuda_server_inject)
    std::thread worker;
    cudaMemPool_t pool = nullptr;   // device frames and job tables (keeps its memory mapped)
    // worker time accounting (vox_cuda_server_stats)
    std::atomic<uint64_t> busy_ns{0}, build_ns{0}, alloc_ns{0}, bytes_out{0}, bytes_full{0};
};

namespace {

// Runs on a driver thread once the launch's work and copies are done.  It
// takes no lock and makes no CUDA call: the worker may hold the server lock
// inside a CUDA call that waits for this stream, so blocking here could
// deadlock.  A missed wake-up costs at most the worker's poll interval.
void CUDART_CB on_launch_done(void *arg)
{
    Launch *L = static_cast<Launch *>(arg);
    vox_cuda_server *s = L->srv;
    L->t_cb.store(now_ns(), std::memory_order_relaxed);
    L->finished.store(true, std::memory_order_release);
    s->cv_work.notify_one();
}

// A launch whose callback is queued is retired only after the callback ran
// (it still touches the launch); otherwise its event is polled.
bool launch_finished(Launch *L)
{
    if (L->has_callback) {
        if (!L->finished.load(std::memory_order_acquire)) return false;
        uint64_t t = L->t_cb.load(std::memory_order_relaxed);
        for (Request *r : L->reqs) if (!r->t_done) r->t_done = t;
        return true;
    }
    if (L->done && cudaEventQuery(L->done) == cudaSuccess) {
        uint64_t t = now_ns();
        for (Request *r : L->reqs) if (!r->t_done) r->t_done = t;
        return true;
    }
    return false;
}

// Under the lock: finished launches leave the in-flight list, their requests
// are published and their memory is returned to the budgets; the buffers
// themselves are handed back later by release_launch, outside the lock.
void retire(vox_cuda_server *s, std::vector<Launch *> &out)
{
    bool any = false;
    for (size_t i = 0; i < s->inflight.size();) {
        Launch *L = s->inflight[i];
        if (!launch_finished(L)) { i++; continue; }
        for (Request *r : L->reqs) {
            if (r->h_in) L->host_free.push_back({r->h_in, r->h_in_cls});
            r->h_in = nullptr;
            if (!r->d_res) r->dev_hold = 0;      // nothing of it stays on the device
            s->used -= r->dev_bytes - r->dev_hold;
            s->host_used -= r->host_bytes;
            s->inflight_reqs--;
            r->done = true;
            s->completed++;
        }
        out.push_back(L);
        s->inflight[i] = s->inflight.back();
        s->inflight.pop_back();
        any = true;
    }
    if (any) s->cv_done.notify_all();
}

// Outside the lock: give a retired launch's buffers back (stream-ordered).
void release_launch(vox_cuda_server *s, Launch *L)
{
    for (auto &hp : L->host_free) s->pinned.put(hp.first, hp.second);
    if (L->d_table) cudaFreeAsync(L->d_table, L->stream);
    if (L->d_frames) cudaFreeAsync(L->d_frames, L->stream);
    s->pinned.put(L->h_table, L->h_table_cls);
    if (L->done) cudaEventDestroy(L->done);
    delete L;
}

// Outside the lock: everything admitted since the last launch, as one launch
// on stream st.  The requests are not yet published, so no client touches
// them meanwhile.
Launch *build_launch(vox_cuda_server *s, const std::vector<Request *> &batch, cudaStream_t st)
{
    const int inj = s->inject.exchange(0);
    if (inj == VOX_CUDA_INJECT_WORKER_FAILURE) throw std::bad_alloc();
    // every allocation that may throw, before any work is enqueued
    std::unique_ptr<Launch> own(new Launch());
    Launch *L = own.get();
    L->srv = s;
    L->stream = st;
    uint64_t t = now_ns();
    std::vector<vox_cuda_frame_job> jobs;
    std::vector<Request *> frames;
    std::vector<size_t> frame_at;   // offset of each frame in the launch's device frames
    L->reqs.reserve(batch.size());
    L->host_free.reserve(batch.size());
    jobs.reserve(batch.size());
    frames.reserve(batch.size());
    frame_at.reserve(batch.size());
    size_t frame_bytes = 0;
    own.release();
    for (Request *r : batch) {
        r->t_launch = t;
        L->reqs.push_back(r);
        if (inj == VOX_CUDA_INJECT_REQUEST_ERROR) {   // as if this launch's enqueue had failed
            r->status = VOX_CUDA_ECUDA;
            continue;
        }
        size_t out_bytes = r->kind == FRAME ? (size_t)r->w * r->h * 4 : (size_t)r->n;
        r->res_bytes = out_bytes;
        const bool on_device = r->kind == FRAME && s->cfg.frames_on_device;
        if (on_device) {   // the frame is drawn where the client will read it
            uint64_t ta = now_ns();
            cudaError_t e = cudaMallocFromPoolAsync(&r->d_res, out_bytes, s->pool, st);
            s->alloc_ns.fetch_add(now_ns() - ta, std::memory_order_relaxed);
            if (e != cudaSuccess) {
                r->d_res = nullptr;
                r->status = VOX_CUDA_ENOMEM;
                continue;
            }
            r->dev_hold = r->dev_bytes - 256;    // the frame; its job-table share goes with the launch
        } else {
            r->h_res = s->pinned.get(out_bytes, &r->h_cls, r->kind == FRAME ? &r->h_dirty : nullptr);
        }
        void *d_res = nullptr;
        if ((!on_device && !r->h_res) ||
            (r->kind != FRAME && cudaHostGetDevicePointer(&d_res, r->h_res, 0) != cudaSuccess)) {
            r->status = VOX_CUDA_ENOMEM;
            continue;
        }
        if (r->kind == FRAME) {
            vox_cuda_frame_job j;
            j.tree = s->trees[r->tree];
            j.camera = r->cam;
            j.w = r->w;
            j.h = r->h;
            j.texture = s->d_tex;
            j.argb = nullptr;   // set once the launch's device frames exist
            jobs.push_back(j);
            frames.push_back(r);
            frame_at.push_back(on_device ? SIZE_MAX : frame_bytes);
            if (!on_device) frame_bytes += (out_bytes + 255) & ~size_t(255);
        } else {
            size_t n = r->n, in_bytes = n * 16;
            void *d_in = nullptr;
            r->h_in = s->pinned.get(in_bytes, &r->h_in_cls);
            if (!r->h_in || cudaHostGetDevicePointer(&d_in, r->h_in, 0) != cudaSuccess) {
                r->status = VOX_CUDA_ENOMEM;
                continue;
            }
            std::memcpy(r->h_in, r->centres.data(), n * 12);
            std::memcpy(static_cast<char *>(r->h_in) + n * 12, r->radii.data(), n * 4);
            const char *d = static_cast<const char *>(d_in);
            int rc = vox_cuda_ball_batch_device(s->trees[r->tree], reinterpret_cast<const float *>(d),
                                                reinterpret_cast<const float *>(d + n * 12), n,
                                                static_cast<uint8_t *>(d_res), st);
            if (rc) r->status = rc;
        }
    }
    if (!jobs.empty()) {
        size_t tb = (frame_job_table_bytes((uint32_t)jobs.size()) + 255) & ~(size_t)255;
        L->h_table = s->pinned.get(tb, &L->h_table_cls);
        int rc = VOX_CUDA_ENOMEM;
        uint64_t ta = now_ns();
        bool got = L->h_table && cudaMallocFromPoolAsync(&L->d_table, tb + 256, s->pool, st) == cudaSuccess &&
                   (frame_bytes == 0 || cudaMallocFromPoolAsync(&L->d_frames, frame_bytes, s->pool, st) == cudaSuccess);
        s->alloc_ns.fetch_add(now_ns() - ta, std::memory_order_relaxed);
        if (got) {
            for (size_t q = 0; q < jobs.size(); q++)
                jobs[q].argb = frame_at[q] == SIZE_MAX
                                   ? static_cast<uint32_t *>(frames[q]->d_res)
                                   : reinterpret_cast<uint32_t *>(static_cast<char *>(L->d_frames) + frame_at[q]);
            uint32_t *counter = reinterpret_cast<uint32_t *>(static_cast<char *>(L->d_table) + tb);
            rc = enqueue_frame_jobs(jobs.data(), (uint32_t)jobs.size(), L->h_table, L->d_table, counter,
                                    s->nsm, st);
            // results out after the kernel: only what differs from what the
            // pinned buffer already holds (the frame is zero outside its
            // tree's screen rectangle, and so is the buffer outside the
            // rectangle of the frame it held last)
            for (size_t q = 0; q < frames.size() && rc == VOX_CUDA_OK; q++) {
                Request *r = frames[q];
                if (r->d_res) continue;                                          // stays on the device
                uint32_t rect[4];
                double centre[2];
                frame_rect_of(s->trees[r->tree], r->cam, r->w, r->h, rect, centre);
                Dirty after;
                const FrameCopy c = plan_frame_copy(r->h_dirty, r->w, r->h, rect, after);
                const size_t pitch = (size_t)r->w * 4;
                size_t moved = 0;
                cudaError_t e = cudaSuccess;
                if (c.full) {
                    moved = r->res_bytes;
                    e = cudaMemcpyAsync(r->h_res, jobs[q].argb, moved, cudaMemcpyDeviceToHost, st);
                } else if (c.x1 > c.x0 && c.y1 > c.y0) {
                    const size_t at = (size_t)c.y0 * pitch + (size_t)c.x0 * 4;
                    moved = (size_t)(c.x1 - c.x0) * 4 * (c.y1 - c.y0);
                    e = cudaMemcpy2DAsync(static_cast<char *>(r->h_res) + at, pitch,
                                          reinterpret_cast<const char *>(jobs[q].argb) + at, pitch,
                                          (size_t)(c.x1 - c.x0) * 4, c.y1 - c.y0, cudaMemcpyDeviceToHost, st);
                }
                if (e != cudaSuccess) rc = VOX_CUDA_ECUDA;
                r->h_dirty = after;
                s->bytes_out.fetch_add(moved, std::memory_order_relaxed);
                s->bytes_full.fetch_add(r->res_bytes, std::memory_order_relaxed);
            }
        }
        if (rc)
            for (Request *r : frames) r->status = rc;
    }
    // completion is seen through the event; the callback only wakes the worker
    if (cudaEventCreateWithFlags(&L->done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventRecord(L->done, st) != cudaSuccess) {
        if (L->done) cudaEventDestroy(L->done);
        L->done = nullptr;
    }
    L->has_callback = cudaLaunchHostFunc(st, on_launch_done, L) == cudaSuccess;
    if (!L->has_callback && !L->done) {
        // neither a callback nor an event: wait for the stream outside any callback path
        cudaStreamSynchronize(st);
        uint64_t t2 = now_ns();
        for (Request *r : L->reqs) { r->t_done = t2; if (!r->status) r->status = VOX_CUDA_ECUDA; }
        L->finished.store(true);
        L->has_callback = true;
    }
    return L;
}

void admit(vox_cuda_server *s)
{
    while (!s->pending.empty()) {
        Request *r = s->pending.front();
        if (s->inflight_reqs >= s->cfg.max_inflight) break;
        if (s->used + r->dev_bytes > s->cfg.budget_bytes) break;   // arrival order: no overtaking
        if (s->host_used + r->host_bytes > s->cfg.host_budget_bytes) break;
        s->pending.pop_front();
        s->used += r->dev_bytes;
        s->host_used += r->host_bytes;
        s->peak = std::max(s->peak, s->used);
        s->host_peak = std::max(s->host_peak, s->host_used);
        s->inflight_reqs++;
        s->admitted.push_back(r);
        if (s->admitted.size() >= s->cfg.max_batch) break;
    }
}

// The worker met a failure it cannot recover from (an allocation that threw):
// once every stream's work has ended, each request not yet done ends with
// VOX_CUDA_ENOMEM -- those of launches that were fully enqueued keep their
// results -- the budgets are given back, and later submissions are refused.
void stop_on_failure(vox_cuda_server *s, std::vector<Request *> &batch)
{
    for (cudaStream_t st : s->streams) cudaStreamSynchronize(st);
    std::lock_guard<std::mutex> lk(s->mu);
    s->failed = true;
    uint64_t t = now_ns();
    auto end = [&](Request *r, bool charged, bool keep_status) {
        if (r->done) return;
        if (!keep_status) r->status = VOX_CUDA_ENOMEM;
        if (!r->d_res) r->dev_hold = 0;          // a kept frame stays charged until released
        if (charged) {
            s->used -= r->dev_bytes - r->dev_hold;
            s->host_used -= r->host_bytes;
            s->inflight_reqs--;
        }
        r->t_done = t;
        r->done = true;
        s->completed++;
    };
    for (Launch *L : s->inflight) {
        for (Request *r : L->reqs) end(r, true, true);
        L->finished.store(true);
    }
    for (Request *r : batch) end(r, true, false);     // taken for a launch that was never enqueued
    batch.clear();
    if (s->building) s->building--;
    for (Request *r : s->admitted) end(r, true, false);
    s->admitted.clear();
    for (Request *r : s->pending) end(r, false, false);
    s->pending.clear();
    s->cv_done.notify_all();
}

void serve(vox_cuda_server *s, std::vector<Launch *> &retired, std::vector<Request *> &batch);

void worker_loop(vox_cuda_server *s)
{
    cudaSetDevice(s->device);
    std::vector<Launch *> retired;
    std::vector<Request *> batch;
    try {
        retired.reserve(s->cfg.max_launches);
        batch.reserve(s->cfg.max_batch);
        serve(s, retired, batch);
    } catch (...) {
        stop_on_failure(s, batch);
    }
}

void serve(vox_cuda_server *s, std::vector<Launch *> &retired, std::vector<Request *> &batch)
{
    for (;;) {
        cudaStream_t st = nullptr;
        bool quit = false;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait_for(lk, std::chrono::microseconds(s->inflight.empty() ? 2000 : 100), [s] {
                if (s->stop) return true;
                for (Launch *L : s->inflight) if (launch_finished(L)) return true;
                return !s->pending.empty() && s->inflight_reqs < s->cfg.max_inflight;
            });
            retire(s, retired);
            quit = s->stop && s->pending.empty() && s->admitted.empty() && s->inflight.empty();
            admit(s);
            if (!s->admitted.empty() && s->inflight.size() + s->building < s->cfg.max_launches) {
                batch.swap(s->admitted);
                st = s->streams[s->next_stream++ % s->streams.size()];
                s->building++;
            }
        }
        uint64_t t0 = now_ns();
        for (Launch *L : retired) release_launch(s, L);
        retired.clear();
        if (!batch.empty()) {
            uint64_t tb = now_ns();
            Launch *L = build_launch(s, batch, st);
            s->build_ns.fetch_add(now_ns() - tb, std::memory_order_relaxed);
            batch.clear();
            std::lock_guard<std::mutex> lk(s->mu);
            s->building--;
            s->inflight.push_back(L);
            s->launches++;
        }
        s->busy_ns.fetch_add(now_ns() - t0, std::memory_order_relaxed);
        if (quit) break;
    }
}

// device bytes a request holds while admitted: a frame's share of the
// launch's job table and the frame it is drawn into (ball inputs and results
// live in pinned host memory)
uint64_t request_bytes(Kind k, uint64_t a, uint64_t b)
{
    return k == FRAME ? 256 + ((a * b * 4 + 255) & ~uint64_t(255)) : 0;
}

// pinned host bytes a request holds while admitted: its result, and for ball
// requests the staged inputs
uint64_t request_host_bytes(Kind k, uint64_t a, uint64_t b)
{
    return k == FRAME ? pinned_class(a * b * 4) : pinned_class(a) + pinned_class(a * 16);
}

}  // namespace

EXPORT int vox_cuda_server_create(const vox_cuda_server_config *config, const uint8_t *texture,
                                  vox_cuda_server **out)
try {
    if (!out || !texture) return VOX_CUDA_EINVAL;
    *out = nullptr;
    // defaults: the configuration that served the mixed load best (20 kHz of
    // requests with frames copied to host memory: frame p99 2-3 ms; with 8
    // streams and 16 launches in flight 3-12 ms, the launch slots filling up)
    vox_cuda_server_config cfg = {40ull << 30, 16ull << 30, 256, 32, 16, 32, 0};
    if (config) cfg = *config;
    if (cfg.budget_bytes == 0 || cfg.host_budget_bytes == 0 || cfg.max_inflight == 0 || cfg.max_batch == 0 ||
        cfg.max_batch > 1024 || cfg.streams == 0 || cfg.streams > 32 || cfg.max_launches == 0)
        return VOX_CUDA_EINVAL;
    vox_cuda_server *s = new (std::nothrow) vox_cuda_server();
    if (!s) return VOX_CUDA_ENOMEM;
    s->cfg = cfg;
    if (cudaGetDevice(&s->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, s->device) != cudaSuccess) {
        delete s;
        return VOX_CUDA_ENODEV;
    }
    // A pool of its own for the launches' frames and job tables that keeps
    // the memory it has mapped (release threshold: the device budget), so
    // a launch after a quiet spell does not map memory again.
    {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = s->device;
        if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess) { delete s; return VOX_CUDA_ENOMEM; }
        uint64_t keep = cfg.budget_bytes;
        cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (cudaMalloc(&s->d_tex, 32768) != cudaSuccess) { cudaMemPoolDestroy(s->pool); delete s; return VOX_CUDA_ENOMEM; }
    if (cudaMemcpy(s->d_tex, texture, 32768, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(s->d_tex);
        cudaMemPoolDestroy(s->pool);
        delete s;
        return VOX_CUDA_ECUDA;
    }
    for (uint32_t i = 0; i < cfg.streams; i++) {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
            cudaFree(s->d_tex);
            cudaMemPoolDestroy(s->pool);
            delete s;
            return VOX_CUDA_ECUDA;
        }
        s->streams.push_back(st);
    }
    try {
        // half the pinned-host budget (at most 8 GiB) pinned now, the rest
        // in slabs as results need it.  Page-locking while requests are
        // served stalls the worker: at 20 kHz each further 128 MiB slab
        // pinned during a trace went with a frame p99 of 15-76 ms, against
        // 1-3 ms for traces that pinned nothing.
        // With frames kept on the device only ball inputs and hits live in
        // pinned memory: an eighth of the budget (at most 1 GiB) then.
        const uint64_t now = cfg.frames_on_device ? std::min<uint64_t>(cfg.host_budget_bytes / 8, uint64_t(1) << 30)
                                                  : std::min<uint64_t>(cfg.host_budget_bytes / 2, uint64_t(8) << 30);
        if (!s->pinned.start(s->device, now, cfg.host_budget_bytes)) {
            vox_cuda_server_destroy(s);
            return VOX_CUDA_ENOMEM;
        }
        // the worker's vectors never grow past these while it runs
        s->admitted.reserve(cfg.max_batch);
        s->inflight.reserve(cfg.max_launches);
        s->worker = std::thread(worker_loop, s);
    } catch (...) {
        vox_cuda_server_destroy(s);
        return VOX_CUDA_ENOMEM;
    }
    *out = s;
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_server_add_tree(vox_cuda_server *s, const vox_cuda_tree *tree, uint32_t *tree_id)
try {
    if (!s || !tree || !tree_id) return VOX_CUDA_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    vox_cuda_tree_info info;
    vox_cuda_tree_get_info(tree, &info);
    if (s->used + info.device_bytes > s->cfg.budget_bytes) return VOX_CUDA_EBUDGET;
    s->trees.push_back(tree);
    s->used += info.device_bytes;          // resident trees count against the budget
    s->tree_bytes += info.device_bytes;
    s->peak = std::max(s->peak, s->used);
    *tree_id = (uint32_t)(s->trees.size() - 1);
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

static int submit(vox_cuda_server *s, Request *r, uint64_t *ticket)
{
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->failed) { delete r; return VOX_CUDA_ENOMEM; }
    if (r->tree >= s->trees.size()) { delete r; return VOX_CUDA_EINVAL; }
    if (s->tree_bytes + r->dev_bytes > s->cfg.budget_bytes || r->host_bytes > s->cfg.host_budget_bytes) {
        s->rejected++;
        delete r;
        return VOX_CUDA_EBUDGET;
    }
    r->ticket = s->next_ticket++;
    r->t_submit = now_ns();
    try {
        s->reqs.emplace(r->ticket, r);
    } catch (...) {
        delete r;
        throw;
    }
    try {
        s->pending.push_back(r);
    } catch (...) {
        s->reqs.erase(r->ticket);
        delete r;
        throw;
    }
    s->submitted++;
    *ticket = r->ticket;
    s->cv_work.notify_one();
    return VOX_CUDA_OK;
}

EXPORT int vox_cuda_server_submit_frame(vox_cuda_server *s, uint32_t tree_id, const vox_cuda_camera *camera,
                                        uint32_t w, uint32_t h, uint64_t *ticket)
try {
    if (!s || !camera || !ticket) return VOX_CUDA_EINVAL;
    if (w == 0 || h == 0 || (w & 0xF) || (h & 0x3)) return VOX_CUDA_EGEOMETRY;
    if (camera->kind != VOX_CUDA_CAMERA_SIMPLE && camera->kind != VOX_CUDA_CAMERA_DOOM) return VOX_CUDA_EINVAL;
    Request *r = new (std::nothrow) Request();
    if (!r) return VOX_CUDA_ENOMEM;
    r->kind = FRAME;
    r->tree = tree_id;
    r->cam = *camera;
    r->w = w;
    r->h = h;
    r->dev_bytes = request_bytes(FRAME, w, h);
    r->host_bytes = s->cfg.frames_on_device ? 0 : request_host_bytes(FRAME, w, h);
    return submit(s, r, ticket);
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_server_submit_balls(vox_cuda_server *s, uint32_t tree_id, const float *centres,
                                        const float *radii, uint32_t n, uint64_t *ticket)
try {
    if (!s || !ticket || n == 0 || !centres || !radii) return VOX_CUDA_EINVAL;
    Request *r = new (std::nothrow) Request();
    if (!r) return VOX_CUDA_ENOMEM;
    r->kind = BALLS;
    r->tree = tree_id;
    r->n = n;
    r->centres.assign(centres, centres + 3 * (size_t)n);
    r->radii.assign(radii, radii + n);
    r->dev_bytes = request_bytes(BALLS, n, 0);
    r->host_bytes = request_host_bytes(BALLS, n, 0);
    return submit(s, r, ticket);
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_server_wait(vox_cuda_server *s, uint64_t ticket, uint32_t timeout_ms)
try {
    if (!s) return VOX_CUDA_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return VOX_CUDA_EINVAL;
    Request *r = it->second;
    if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [r] { return r->done; }))
        return VOX_CUDA_ETIMEOUT;
    return r->status;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_server_result(vox_cuda_server *s, uint64_t ticket, const void **data, size_t *bytes,
                                  uint64_t *times_ns)
try {
    if (!s) return VOX_CUDA_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return VOX_CUDA_EINVAL;
    Request *r = it->second;
    if (!r->done) return VOX_CUDA_ETIMEOUT;
    if (data) *data = r->d_res ? r->d_res : r->h_res;
    if (bytes) *bytes = r->res_bytes;
    if (times_ns) {
        times_ns[0] = r->t_submit;
        times_ns[1] = r->t_launch;
        times_ns[2] = r->t_done;
    }
    return r->status;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_server_release(vox_cuda_server *s, uint64_t ticket)
try {
    if (!s) return VOX_CUDA_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return VOX_CUDA_EINVAL;
    Request *r = it->second;
    if (!r->done) return VOX_CUDA_EINVAL;
    // a frame copied without error leaves its buffer in a known state
    s->pinned.put(r->h_res, r->h_cls, r->status == VOX_CUDA_OK ? r->h_dirty : Dirty{});
    if (r->d_res) {   // its launch has ended: the frame is free on any stream
        cudaFreeAsync(r->d_res, s->streams[0]);
        s->used -= r->dev_hold;
    }
    s->reqs.erase(it);
    delete r;
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_server_inject(vox_cuda_server *s, int what)
try {
    if (!s || (what != VOX_CUDA_INJECT_REQUEST_ERROR && what != VOX_CUDA_INJECT_WORKER_FAILURE))
        return VOX_CUDA_EINVAL;
    s->inject.store(what);
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_server_get_stats(vox_cuda_server *s, vox_cuda_server_stats *st)
try {
    if (!s || !st) return VOX_CUDA_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    st->submitted = s->submitted;
    st->completed = s->completed;
    st->rejected = s->rejected;
    st->launches = s->launches;
    st->bytes_in_use = s->used;
    st->peak_bytes = s->peak;
    st->pending = s->pending.size();
    st->inflight = s->inflight_reqs;
    st->host_bytes_in_use = s->host_used;
    st->host_peak_bytes = s->host_peak;
    st->worker_busy_ns = s->busy_ns.load();
    st->build_ns = s->build_ns.load();
    st->host_pin_ns = s->pinned.pin_ns.load();
    st->host_pins = s->pinned.pins.load();
    st->device_alloc_ns = s->alloc_ns.load();
    st->frame_bytes_out = s->bytes_out.load();
    st->host_slabs = s->pinned.slabs();
    st->frame_bytes_full = s->bytes_full.load();
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_server_destroy(vox_cuda_server *s)
try {
    if (!s) return VOX_CUDA_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_one();
    if (s->worker.joinable()) s->worker.join();
    for (Launch *L : s->inflight) release_launch(s, L);   // left by a worker stopped on a failure
    s->inflight.clear();
    for (auto &kv : s->reqs)
        if (kv.second->d_res) {
            cudaFreeAsync(kv.second->d_res, s->streams[0]);
            kv.second->d_res = nullptr;
        }
    for (cudaStream_t st : s->streams) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    for (auto &kv : s->reqs) {
        s->pinned.put(kv.second->h_res, kv.second->h_cls);
        delete kv.second;
    }
    cudaFree(s->d_tex);
    if (s->pool) cudaMemPoolDestroy(s->pool);   // every launch's memory was freed on its synchronised stream
    delete s;
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

/* ---------------------------------------------------------------------------
 * Trace replay: a request trace submitted at its arrival times from a native
 * thread, completions collected by `collectors` threads that wait on the
 * tickets in arrival order and release them.  The submitting thread sleeps
 * until shortly before each arrival and spins the rest, so arrivals keep
 * their spacing at tens of kHz; per-request times are the server's own.
 * ------------------------------------------------------------------------- */

EXPORT int vox_cuda_server_replay(vox_cuda_server *s, const vox_cuda_replay_request *reqs, uint32_t n,
                                  uint32_t collectors, vox_cuda_replay_result *out)
try {
    if (!s || (n && (!reqs || !out)) || collectors == 0 || collectors > 64) return VOX_CUDA_EINVAL;
    for (uint32_t i = 0; i < n; i++) {
        const vox_cuda_replay_request &q = reqs[i];
        if (q.kind > 1 || !(q.arrival_s >= 0.0) || (i && q.arrival_s < reqs[i - 1].arrival_s))
            return VOX_CUDA_EINVAL;
        if (q.kind == 1 && (!q.centres || !q.radii || q.n == 0)) return VOX_CUDA_EINVAL;
    }
    std::vector<std::atomic<uint64_t>> tickets(n);     // 0: not submitted yet
    std::vector<std::atomic<int>> submit_rc(n);
    for (uint32_t i = 0; i < n; i++) { tickets[i].store(0); submit_rc[i].store(VOX_CUDA_OK); out[i] = {}; }
    std::atomic<uint32_t> next{0};
    auto collect = [&]() {
        for (;;) {
            uint32_t i = next.fetch_add(1);
            if (i >= n) return;
            uint64_t tk = 0;
            // wait for the submitter to reach request i (it always does, or
            // records why it could not)
            while ((tk = tickets[i].load(std::memory_order_acquire)) == 0 && submit_rc[i].load() == VOX_CUDA_OK)
                std::this_thread::sleep_for(std::chrono::microseconds(20));
            if (tk == 0) { out[i].status = submit_rc[i].load(); continue; }
            int rc = VOX_CUDA_ETIMEOUT;
            for (int k = 0; k < 600 && rc == VOX_CUDA_ETIMEOUT; k++)   // at most 10 minutes
                rc = vox_cuda_server_wait(s, tk, 1000);
            uint64_t times[3] = {0, 0, 0};
            if (rc != VOX_CUDA_ETIMEOUT) {
                vox_cuda_server_result(s, tk, nullptr, nullptr, times);
                vox_cuda_server_release(s, tk);
            }
            out[i].status = rc;
            out[i].submit_ns = times[0];
            out[i].launch_ns = times[1];
            out[i].done_ns = times[2];
        }
    };
    std::vector<std::thread> pool;
    try {
        for (uint32_t c = 0; c < collectors; c++) pool.emplace_back(collect);
    } catch (...) {
        // fewer collectors; with none, this thread collects after submitting
    }
    const uint64_t t0 = now_ns();
    for (uint32_t i = 0; i < n; i++) {
        const vox_cuda_replay_request &q = reqs[i];
        const uint64_t due = t0 + (uint64_t)(q.arrival_s * 1e9);
        for (;;) {
            uint64_t t = now_ns();
            if (t >= due) break;
            if (due - t > 200000) std::this_thread::sleep_for(std::chrono::nanoseconds(due - t - 100000));
        }
        uint64_t tk = 0;
        int rc = q.kind == 0 ? vox_cuda_server_submit_frame(s, q.tree_id, &q.camera, q.w, q.h, &tk)
                             : vox_cuda_server_submit_balls(s, q.tree_id, q.centres, q.radii, q.n, &tk);
        if (rc) submit_rc[i].store(rc);
        else tickets[i].store(tk, std::memory_order_release);
    }
    if (pool.empty()) collect();
    for (auto &th : pool) th.join();
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT
