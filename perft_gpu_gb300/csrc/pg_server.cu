// pg_server.cu -- continuous-batching perft server (host scheduler + kernels).
//
// A request is (position, depth).  At admission a request deeper than
// TASK_DEPTH is expanded on the GPU into its positions TASK_DEPTH plies above
// the leaves ("tasks"); the tasks stay in a device frontier pool until they
// are counted, so a request's frontier lives on the device for its whole
// life.  Admission is gated by free request slots and by free space in the
// pool (the server's HBM budget).  The scheduler thread runs waves: each wave
// takes one task of every active request (a request admitted a moment ago
// gets work in the very next wave, whatever deep requests are running), then
// fills its budget by least remaining work first, runs the tasks as one
// batched engine call that adds each task's count into its request's device
// counter, and completes the requests whose last task was in the wave.  New
// requests join at every wave boundary, so their work overlaps on the device
// with the running ones.  Waves are sized in time: after every wave the
// scheduler knows each request's leaves per task so far (its counter / its
// tasks run) and the device's leaves per second, and the next wave takes
// about WAVE_SECONDS of work, so a request that arrives while deep ones run
// waits a few milliseconds, not the length of a large wave.
//
// The reference has no serving path; its nearest caller is the host work
// queue of perft_multi_threaded_gpu_launcher (launcher.h:476-583), which
// hands whole root moves to idle GPUs.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pg_engine.cuh"
#include "pg_level.cuh"
#include "pg_tt.cuh"

namespace pg {
namespace {

constexpr int TASK_DEPTH = 5;               // remaining depth of one task
constexpr u32 MAX_WAVE_TASKS = 1u << 16;
#ifndef PG_WAVE_SECONDS
#define PG_WAVE_SECONDS 0.004
#endif
constexpr double WAVE_SECONDS = PG_WAVE_SECONDS;  // target device time of one wave
constexpr double MIN_WAVE_LEAVES = 1e9;     // floor of the timed wave budget
constexpr double MAX_WAVE_LEAVES = 4e10;

struct Segment {
    u64 src;    // first task in the pool (index in boards)
    u32 count;
    u32 dst;    // first slot in the wave
    u32 group;  // request slot
    u32 depth;
};

__global__ void k_gather_wave(const Pos* __restrict__ pool, const Segment* __restrict__ segs, u32 nseg, u32 total,
                              Pos* __restrict__ out, unsigned char* __restrict__ dep, u32* __restrict__ grp)
{
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        u32 lo = 0, hi = nseg - 1;  // last segment with dst <= i
        while (lo < hi) {
            const u32 mid = (lo + hi + 1) / 2;
            if (segs[mid].dst <= i) lo = mid; else hi = mid - 1;
        }
        const Segment s = segs[lo];
        out[i] = pool[s.src + (i - s.dst)];
        dep[i] = (unsigned char)s.depth;
        grp[i] = s.group;
    }
}

// TT waves: add each task's count into its request's counter.  A request's
// tasks form runs of adjacent wave slots (one run per segment); a warp numbers
// the runs among its lanes, sums each run with a segmented shuffle reduction
// and adds it with one atomic.
__global__ void k_add_groups(const u64* __restrict__ task_out, const u32* __restrict__ grp, u32 total,
                             u64* __restrict__ acc)
{
    constexpr unsigned FULL = 0xFFFFFFFFu;
    const u32 lane = threadIdx.x & 31;
    const u32 stride = gridDim.x * blockDim.x;  // a multiple of 32
    for (u32 base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < total; base += stride) {
        const u32 i = base + lane;
        const bool valid = i < total;
        const u32 g = valid ? grp[i] : 0xFFFFFFFFu;
        u64 v = valid ? task_out[i] : 0;
        const u32 prev = __shfl_up_sync(FULL, g, 1);
        const bool head = lane == 0 || prev != g;
        const u32 heads = __ballot_sync(FULL, head);
        const u32 run = __popc(heads & (0xFFFFFFFFu >> (31 - lane)));  // runs up to and including this lane
        for (u32 o = 1; o < 32; o <<= 1) {
            const u64 vn = __shfl_down_sync(FULL, v, o);
            const u32 rn = __shfl_down_sync(FULL, run, o);
            if (lane + o < 32 && rn == run) v += vn;
        }
        if (valid && head) atomicAdd(&acc[g], v);
    }
}

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    Pos pos;
    int depth = 0;
    double t_submit = 0, t_done = 0;
    u64 result = 0;
    int status = PG_OK;
    bool done = false;
    // in flight
    int slot = -1;
    u64 pool_off = 0, pool_len = 0;
    u32 ntasks = 0, next = 0;
    int task_depth = 0;
    u64 acc_seen = 0;     // the request's counter after the last wave
    double per_task = 0;  // measured leaves per task (0 until a wave ran)
    u64 need = 0;         // frontier boards known to be needed (after a deferred admission)
};

// first-fit allocator over the frontier pool (units: boards)
struct PoolAlloc {
    std::map<u64, u64> free_;  // offset -> length
    void reset(u64 cap)
    {
        free_.clear();
        if (cap) free_[0] = cap;
    }
    u64 largest() const
    {
        u64 m = 0;
        for (const auto& kv : free_) m = std::max(m, kv.second);
        return m;
    }
    bool take_largest(u64& off, u64& len)
    {
        auto best = free_.end();
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (best == free_.end() || it->second > best->second) best = it;
        if (best == free_.end()) return false;
        off = best->first;
        len = best->second;
        free_.erase(best);
        return true;
    }
    void give(u64 off, u64 len)
    {
        if (!len) return;
        auto it = free_.emplace(off, len).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

struct Server {
    std::mutex mu;  // guards the request table and the queues
    std::condition_variable cv;
    std::thread th;
    bool running = false;
    u64 next_id = 1;
    std::unordered_map<u64, Request> reqs;
    std::deque<u64> pending;
    std::vector<u64> active;  // admission order
    std::vector<int> free_slots;
    u32 max_inflight = 4096;
    int slider = 0;
    int use_tt = PG_TT_OFF;  // pg_tt_mode of the waves
    bool persistent = false;  // waves as one persistent launch
    u64 tt_bytes = 0;
    double wave_leaves = 4e9;  // fixed wave budget (max_wave_nodes) or the first wave's
    bool timed_waves = true;   // size waves from the measured rate
    double rate = 0;           // leaves per second over recent waves
    // device
    u64* acc = nullptr;
    Pos* pool = nullptr;
    u64 pool_cap = 0;
    PoolAlloc alloc;
    Pos* wave_pos = nullptr;
    unsigned char* wave_dep = nullptr;
    u32* wave_grp = nullptr;
    u64* task_out = nullptr;      // per-task counts of a TT wave
    Segment* seg_dev = nullptr;
    Segment* seg_host = nullptr;  // pinned
    u64* acc_host = nullptr;      // pinned
    // statistics
    u64 waves = 0;
    u64 submitted = 0, completed = 0, deferred = 0;
    u32 max_active = 0;
    u64 pool_used = 0, pool_peak = 0;
};

Server* g_srv = nullptr;

double est_leaves(int d)
{
    static const double t[16] = {1, 30, 900, 2.7e4, 8.1e5, 2.4e7, 7.3e8, 2.2e10, 6.6e11, 2e13, 6e14, 1.8e16,
                                 5e17, 1.5e19, 4.5e20, 1.3e22};
    return t[std::min(std::max(d, 0), 15)];
}

#define SRV_CUDA(call)                                                         \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            set_error("%s failed: %s", #call, cudaGetErrorString(e_));         \
            return PG_ERR_CUDA;                                                \
        }                                                                      \
    } while (0)

void finish(Server& S, Request& r, int status, u64 result)
{
    S.completed++;
    r.status = status;
    r.result = result;
    r.t_done = now_s();
    r.done = true;
}

// admit pending requests while slots and pool space allow (engine mutex held)
void admit(Server& S, std::unique_lock<std::mutex>& lk)
{
    while (!S.pending.empty() && !S.free_slots.empty()) {
        const u64 id = S.pending.front();
        Request& r = S.reqs[id];
        if (r.need > S.pool_cap) {  // can never fit the pool
            S.pending.pop_front();
            set_error("request needs %llu frontier positions, over the pool of %llu", (unsigned long long)r.need,
                      (unsigned long long)S.pool_cap);
            finish(S, r, PG_ERR_CAPACITY, 0);
            continue;
        }
        // a request that did not fit waits (first in line: no starvation)
        // until a free block holds what it is known to need
        if (r.need && S.alloc.largest() < r.need) return;
        u64 off = 0, len = 0;
        if (!S.alloc.take_largest(off, len)) return;  // pool full: wait for frees
        const int plies = r.depth > TASK_DEPTH ? r.depth - TASK_DEPTH : 0;
        u32 n = 0;
        int st = PG_OK;
        if (plies == 0) {
            if (cudaMemcpyAsync(S.pool + off, &r.pos, sizeof(Pos), cudaMemcpyHostToDevice, engine().stream) != cudaSuccess ||
                cudaStreamSynchronize(engine().stream) != cudaSuccess)
                st = PG_ERR_CUDA;
            n = 1;
        } else {
            lk.unlock();
            const u32 cap = (u32)std::min<u64>(len, 0xFFFFFFFFull);
            st = expand_frontier(r.pos, plies, S.pool + off, cap, &n);
            lk.lock();
        }
        if (st == PG_ERR_CAPACITY && !S.active.empty()) {
            S.alloc.give(off, len);  // retry once running requests release memory
            r.need = std::max<u64>(r.need, (u64)n + 1 > len ? (u64)n : len + 1);
            S.deferred++;
            return;
        }
        S.pending.pop_front();
        if (st != PG_OK) {
            S.alloc.give(off, len);
            finish(S, r, st, 0);
            continue;
        }
        if (n == 0) {  // no legal continuation before the task depth
            S.alloc.give(off, len);
            finish(S, r, PG_OK, 0);
            continue;
        }
        S.alloc.give(off + n, len - n);
        S.pool_used += n;
        S.pool_peak = std::max(S.pool_peak, S.pool_used);
        r.slot = S.free_slots.back();
        S.free_slots.pop_back();
        r.pool_off = off;
        r.pool_len = n;
        r.ntasks = n;
        r.next = 0;
        r.task_depth = plies ? TASK_DEPTH : r.depth;
        S.active.push_back(id);
        S.max_active = std::max<u32>(S.max_active, (u32)S.active.size());
    }
}

// one wave over the active requests (engine mutex held, server mutex held)
int run_wave(Server& S, std::unique_lock<std::mutex>& lk)
{
    Engine& E = engine();
    std::vector<Segment> segs;
    u32 total = 0;
    const double wave_leaves =
        (S.timed_waves && S.rate > 0)
            ? std::min(MAX_WAVE_LEAVES, std::max(MIN_WAVE_LEAVES, S.rate * WAVE_SECONDS))
            : S.wave_leaves;
    // pass 1: one task of every active request, so none waits for a whole
    // wave; pass 2: the rest of the budget by least remaining work first
    // (a request's remaining tasks x its measured leaves per task), which
    // keeps short requests from queueing behind long ones
    double budget = wave_leaves;
    std::vector<std::pair<double, u64>> order;
    order.reserve(S.active.size());
    for (u64 id : S.active) {
        Request& r = S.reqs[id];
        if (r.next >= r.ntasks || total >= MAX_WAVE_TASKS) continue;
        const double per = r.per_task > 0 ? r.per_task : est_leaves(r.task_depth);
        segs.push_back(Segment{r.pool_off + r.next, 1u, total, (u32)r.slot, (u32)r.task_depth});
        r.next += 1;
        total += 1;
        budget -= per;
        order.emplace_back(per * (r.ntasks - r.next), id);
    }
    std::sort(order.begin(), order.end());
    for (const auto& o : order) {
        if (budget <= 0 || total >= MAX_WAVE_TASKS) break;
        Request& r = S.reqs[o.second];
        if (r.next >= r.ntasks) continue;
        const double per = r.per_task > 0 ? r.per_task : est_leaves(r.task_depth);
        u32 k = (u32)std::min<double>(budget / per + 1.0, (double)(r.ntasks - r.next));
        k = std::min(k, MAX_WAVE_TASKS - total);
        if (k == 0) continue;
        segs.push_back(Segment{r.pool_off + r.next, k, total, (u32)r.slot, (u32)r.task_depth});
        r.next += k;
        total += k;
        budget -= k * per;
    }
    if (!total) return PG_OK;
    const double t_wave = now_s();
    memcpy(S.seg_host, segs.data(), segs.size() * sizeof(Segment));
    SRV_CUDA(cudaMemcpyAsync(S.seg_dev, S.seg_host, segs.size() * sizeof(Segment), cudaMemcpyHostToDevice, E.stream));
    k_gather_wave<<<std::min<u32>((total + 255) / 256, 2048), 256, 0, E.stream>>>(S.pool, S.seg_dev, (u32)segs.size(),
                                                                                 total, S.wave_pos, S.wave_dep,
                                                                                 S.wave_grp);
    SRV_CUDA(cudaGetLastError());
    lk.unlock();
    E.ticket_next = 0;
    cudaMemsetAsync(E.tickets, 0, MAX_TICKETS * sizeof(u32), E.stream);
    cudaMemsetAsync(E.err, 0, sizeof(u32), E.stream);
    pg_opts o{};
    o.slider = S.slider;
    int st;
    if (S.use_tt) {
        o.use_tt = S.use_tt;
        o.tt_bytes = S.tt_bytes;
        st = tt_perft_batch_device(S.wave_pos, S.wave_dep, total, S.task_out, &o);
        if (st == PG_OK) {
            k_add_groups<<<std::min<u32>((total + 255) / 256, 2048), 256, 0, E.stream>>>(S.task_out, S.wave_grp,
                                                                                       total, S.acc);
            if (cudaGetLastError() != cudaSuccess) st = PG_ERR_CUDA;
        }
    } else if (S.persistent) {
        int maxd = 0;
        for (const Segment& sg : segs) maxd = std::max<int>(maxd, (int)sg.depth);
        st = perft_core_persistent(S.wave_pos, S.wave_dep, S.wave_grp, total, S.acc, false, maxd);
    } else {
        st = perft_core(S.wave_pos, S.wave_dep, S.wave_grp, total, S.acc, false, pick_variant(&o));
    }
    if (st == PG_OK) {
        if (cudaMemcpyAsync(S.acc_host, S.acc, S.max_inflight * sizeof(u64), cudaMemcpyDeviceToHost, E.stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(E.stream) != cudaSuccess)
            st = PG_ERR_CUDA;
    }
    lk.lock();
    S.waves++;
    if (st == PG_OK) {
        // measured leaves per task of every request and the device's rate
        double got = 0;
        for (u64 id : S.active) {
            Request& r = S.reqs[id];
            const u64 a = S.acc_host[r.slot];
            got += (double)(a - r.acc_seen);
            r.acc_seen = a;
            if (r.next) r.per_task = std::max(1.0, (double)a / r.next);
        }
        const double dt = now_s() - t_wave;
        if (dt > 0 && got > 0) S.rate = S.rate > 0 ? 0.5 * S.rate + 0.5 * got / dt : got / dt;
    }
    // completions
    std::vector<u64> still;
    for (u64 id : S.active) {
        Request& r = S.reqs[id];
        if (st != PG_OK) {
            finish(S, r, st, 0);
        } else if (r.next >= r.ntasks) {
            finish(S, r, PG_OK, S.acc_host[r.slot]);
        } else {
            still.push_back(id);
            continue;
        }
        cudaMemsetAsync(S.acc + r.slot, 0, sizeof(u64), E.stream);
        S.free_slots.push_back(r.slot);
        S.alloc.give(r.pool_off, r.pool_len);
        S.pool_used -= r.pool_len;
        r.slot = -1;
    }
    S.active.swap(still);
    return st;
}

void server_loop(Server& S)
{
    Engine& E = engine();
    std::unique_lock<std::mutex> lk(S.mu);
    while (S.running) {
        if (S.pending.empty() && S.active.empty()) {
            S.cv.wait_for(lk, std::chrono::milliseconds(50));
            continue;
        }
        lk.unlock();
        std::unique_lock<std::mutex> eng(E.mu);
        lk.lock();
        admit(S, lk);
        if (!S.active.empty()) run_wave(S, lk);
        eng.unlock();
        S.cv.notify_all();
    }
}

void release(Server* S)
{
    if (S->acc) cudaFree(S->acc);
    if (S->pool) cudaFree(S->pool);
    if (S->wave_pos) cudaFree(S->wave_pos);
    if (S->wave_dep) cudaFree(S->wave_dep);
    if (S->wave_grp) cudaFree(S->wave_grp);
    if (S->task_out) cudaFree(S->task_out);
    if (S->seg_dev) cudaFree(S->seg_dev);
    if (S->seg_host) cudaFreeHost(S->seg_host);
    if (S->acc_host) cudaFreeHost(S->acc_host);
    delete S;
}

}  // namespace
}  // namespace pg

using namespace pg;

extern "C" {

int pg_server_start(const pg_server_config* cfg)
{
    Engine& E = engine();
    {
        std::lock_guard<std::mutex> lk(E.mu);
        if (!E.ready) {
            set_error("pg_init has not been called");
            return PG_ERR_NOT_INITIALIZED;
        }
    }
    if (g_srv) {
        set_error("server already running");
        return PG_ERR_BUSY;
    }
    Server* S = new Server();
    S->max_inflight = (cfg && cfg->max_inflight) ? cfg->max_inflight : 4096;
    S->slider = cfg ? cfg->slider : 0;
    S->use_tt = cfg ? cfg->use_tt : PG_TT_OFF;
    if (S->use_tt < PG_TT_OFF || S->use_tt > PG_TT_DEDUP_ONLY) {
        delete S;
        set_error("use_tt %d is not a pg_tt_mode", cfg->use_tt);
        return PG_ERR_INVALID_ARGUMENT;
    }
    S->tt_bytes = cfg ? cfg->tt_bytes : 0;
    S->persistent = cfg && cfg->persistent;
    if (cfg && cfg->max_wave_nodes) {
        S->wave_leaves = (double)cfg->max_wave_nodes * est_leaves(TASK_DEPTH);
        S->timed_waves = false;
    }
    const u64 budget = (cfg && cfg->hbm_budget_bytes) ? cfg->hbm_budget_bytes : (2ull << 30);
    S->pool_cap = budget / sizeof(Pos);
    cudaError_t e = cudaSetDevice(E.device);
    if (e == cudaSuccess) e = cudaMalloc(&S->acc, S->max_inflight * sizeof(u64));
    if (e == cudaSuccess) e = cudaMemset(S->acc, 0, S->max_inflight * sizeof(u64));
    // the engine's kernels run on a non-blocking stream: finish the clear here
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e == cudaSuccess) e = cudaMalloc(&S->pool, S->pool_cap * sizeof(Pos));
    if (e == cudaSuccess) e = cudaMalloc(&S->wave_pos, MAX_WAVE_TASKS * sizeof(Pos));
    if (e == cudaSuccess) e = cudaMalloc(&S->wave_dep, MAX_WAVE_TASKS);
    if (e == cudaSuccess) e = cudaMalloc(&S->wave_grp, MAX_WAVE_TASKS * sizeof(u32));
    if (e == cudaSuccess && S->use_tt) e = cudaMalloc(&S->task_out, MAX_WAVE_TASKS * sizeof(u64));
    if (e == cudaSuccess) e = cudaMalloc(&S->seg_dev, (S->max_inflight * 2 + 8) * sizeof(Segment));
    if (e == cudaSuccess) e = cudaMallocHost(&S->seg_host, (S->max_inflight * 2 + 8) * sizeof(Segment));
    if (e == cudaSuccess) e = cudaMallocHost(&S->acc_host, S->max_inflight * sizeof(u64));
    if (e != cudaSuccess) {
        set_error("server allocation failed: %s", cudaGetErrorString(e));
        release(S);
        return e == cudaErrorMemoryAllocation ? PG_ERR_OUT_OF_MEMORY : PG_ERR_CUDA;
    }
    S->alloc.reset(S->pool_cap);
    for (int i = (int)S->max_inflight - 1; i >= 0; i--) S->free_slots.push_back(i);
    S->running = true;
    g_srv = S;
    S->th = std::thread(server_loop, std::ref(*S));
    return PG_OK;
}

int pg_server_submit(const pg_board* pos, int depth, uint64_t* request_id)
{
    Server* S = g_srv;
    if (!S) {
        set_error("server not running");
        return PG_ERR_NOT_INITIALIZED;
    }
    if (!pos || !request_id || depth < 0 || depth > 15) {
        set_error("bad argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    const u64 inner = INNER;
    const u64 pawns = pos->pawns & inner;
    const u64 occ = pawns | pos->knights | pos->bishop_queens | pos->rook_queens | pos->kings;
    if ((pawns & (pos->knights | pos->bishop_queens | pos->rook_queens | pos->kings)) ||
        (pos->knights & (pos->bishop_queens | pos->rook_queens | pos->kings)) ||
        ((pos->bishop_queens | pos->rook_queens) & pos->kings) || (pos->white & ~occ) ||
        __builtin_popcountll(pos->kings & pos->white) != 1 || __builtin_popcountll(pos->kings & ~pos->white) != 1) {
        set_error("not a valid board");
        return PG_ERR_INVALID_POSITION;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    const u64 id = S->next_id++;
    Request& r = S->reqs[id];
    memcpy(&r.pos, pos, sizeof(Pos));
    r.depth = depth;
    r.t_submit = now_s();
    S->submitted++;
    S->pending.push_back(id);
    *request_id = id;
    S->cv.notify_all();
    return PG_OK;
}

int pg_server_poll(uint64_t request_id, uint64_t* result, int* done, double* latency_ms)
{
    Server* S = g_srv;
    if (!S) {
        set_error("server not running");
        return PG_ERR_NOT_INITIALIZED;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(request_id);
    if (it == S->reqs.end()) {
        set_error("unknown request %llu", (unsigned long long)request_id);
        return PG_ERR_INVALID_ARGUMENT;
    }
    const Request& r = it->second;
    if (done) *done = r.done ? 1 : 0;
    if (r.done) {
        if (result) *result = r.result;
        if (latency_ms) *latency_ms = 1e3 * (r.t_done - r.t_submit);
        if (r.status != PG_OK) {
            set_error("request %llu failed with status %d", (unsigned long long)request_id, r.status);
            return r.status;
        }
    }
    return PG_OK;
}

int pg_server_get_stats(pg_server_stats* out)
{
    Server* S = g_srv;
    if (!S) {
        set_error("server not running");
        return PG_ERR_NOT_INITIALIZED;
    }
    if (!out) {
        set_error("null argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    out->submitted = S->submitted;
    out->completed = S->completed;
    out->waves = S->waves;
    out->admissions_deferred = S->deferred;
    out->max_active = S->max_active;
    out->pool_capacity = S->pool_cap;
    out->pool_peak = S->pool_peak;
    return PG_OK;
}

int pg_server_stop(void)
{
    Server* S = g_srv;
    if (!S) return PG_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->running = false;
        S->cv.notify_all();
    }
    S->th.join();
    {
        std::lock_guard<std::mutex> lk(engine().mu);
        cudaStreamSynchronize(engine().stream);
        g_srv = nullptr;
        release(S);
    }
    return PG_OK;
}

}  // extern "C"
