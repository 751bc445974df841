// pg_engine.cu -- launch plans, the chunked breadth-first
// driver and the C ABI of the GB300 perft engine.
//
// Host-side control follows the reference's no-TT launcher
// (perftLauncher, launcher.h:1467-1503; perft_bb_gpu_simple,
// perft_bb.h:1027-1138) but without dynamic parallelism: the host walks the
// levels, a level that would not fit its buffer is split into chunks that do
// (the reference instead picks a launch depth from a branching-factor
// estimate, launcher.h:1535-1563), and every wait on the device is bounded.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "pg_engine.cuh"
#include "pg_level.cuh"
#include "pg_ops.cuh"
#include "pg_tt.cuh"

namespace pg {

static Engine g_engine;
Engine& engine() { return g_engine; }

static thread_local std::string t_error;

void set_error(const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_error = buf;
}

#define PG_CUDA(call)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? PG_ERR_OUT_OF_MEMORY : PG_ERR_CUDA;    \
        }                                                                                    \
    } while (0)

#define PG_TRY(expr)              \
    do {                          \
        int r_ = (expr);          \
        if (r_ != PG_OK) return r_; \
    } while (0)

// ---------------------------------------------------------------------------
// launch plans
// ---------------------------------------------------------------------------

u32* next_ticket()
{
    Engine& E = engine();
    if (E.ticket_next >= MAX_TICKETS - 8) return nullptr;
    return E.tickets + E.ticket_next++;
}

#define PG_TICKET(var)                              \
    u32* var = next_ticket();                       \
    if (!var) {                                     \
        set_error("dynamic-scheduling counters exhausted"); \
        return PG_ERR_CAPACITY;                     \
    }

int launch_leaf(const Variant& v, int side, const LevelView& lv, u32 start, u32 n, u64* acc)
{
    Engine& E = engine();
    PG_TICKET(tk);
    PG_CUDA(ops_for(v.slider).leaf(side, v.T, lv, start, n, acc, tk, (u32)v.leaf_plies, E.stream, E.num_sms));
    E.st.launches++;
    E.st.leaf_kernel_launches++;
    E.st.leaf_parent_nodes += n;
    return PG_OK;
}

int launch_expand(const Variant& v, int side, const LevelView& in, u32 start, u32 a, u32 b, const u64* offs,
                         const LevelView& out)
{
    Engine& E = engine();
    PG_TICKET(tk);
    PG_CUDA(ops_for(v.slider).expand(side, v.T, in, start, a, b, offs, out, tk, E.stream, E.num_sms));
    E.st.launches++;
    return PG_OK;
}

int launch_count(const Variant& v, int side, const LevelView& lv, u32 start, u32 n, u32* cnt)
{
    Engine& E = engine();
    PG_CUDA(ops_for(v.slider).count_level(side, lv, start, n, cnt, (u32)v.leaf_plies + 1, E.stream, E.num_sms));
    E.st.launches++;
    return PG_OK;
}

int launch_scan(const u32* cnt, u32 n, u64* offs)
{
    Engine& E = engine();
    const u64 tiles = (n + SCAN_TILE - 1) / SCAN_TILE + 1;
    if (tiles > E.scan_status_cap) {
        E.alloc_gen++;
        if (E.scan_status) cudaFree(E.scan_status);
        E.scan_status = nullptr;
        E.scan_status_cap = 0;
        PG_CUDA(cudaMalloc(&E.scan_status, tiles * sizeof(u64)));
        E.scan_status_cap = tiles;
    }
    u32* tk = next_ticket();
    if (!tk) {
        set_error("ticket pool exhausted");
        return PG_ERR_CAPACITY;
    }
    PG_CUDA(cudaMemsetAsync(E.scan_status, 0, tiles * sizeof(u64), E.stream));
    const u32 grid = (u32)std::max<u64>(1, (n + SCAN_TILE - 1) / SCAN_TILE);
    k_scan<<<grid, SCAN_T, 0, E.stream>>>(cnt, n, offs, E.scan_status, tk, E.err);
    PG_CUDA(cudaGetLastError());
    E.st.launches++;
    return PG_OK;
}

// ---------------------------------------------------------------------------
// level buffers
// ---------------------------------------------------------------------------

static constexpr u64 NODE_BYTES = LEVEL_NODE_BYTES;

u64 level_cap_max()
{
    Engine& E = engine();
    u64 cap = E.budget / NODE_BYTES / 4;
    cap = std::min<u64>(cap, 0xF0000000ull);
    return std::max<u64>(cap, 1u << 16);
}

int ensure_level(int L, u64 need)
{
    Engine& E = engine();
    if (L >= MAX_LEVELS) {
        set_error("depth exceeds %d levels", MAX_LEVELS);
        return PG_ERR_CAPACITY;
    }
    LevelBuf& lb = E.lv[L];
    if (lb.cap >= need) return PG_OK;
    // rounded up to an eighth of the next power of two (at most 12.5% over
    // the need, so a level regrows rarely without doubling its bytes)
    u64 p2 = 1u << 16;
    while (p2 < need) p2 <<= 1;
    const u64 step = std::max<u64>(p2 / 8, 1u << 16);
    u64 cap = (need + step - 1) / step * step;
    cap = std::min(cap, std::max(level_cap_max(), need));
    E.alloc_gen++;
    if (lb.block) {
        PG_CUDA(cudaStreamSynchronize(E.stream));
        cudaFree(lb.block);
        E.level_bytes_total -= lb.cap * NODE_BYTES;
        lb = LevelBuf{};
    }
    const u64 bytes = cap * 48 + cap * 4 + cap + 16 + cap * 4 + (cap + 1) * 8 + 256;
    void* blk = nullptr;
    cudaError_t e = E.fail_next_alloc ? cudaErrorMemoryAllocation : cudaMalloc(&blk, bytes);
    E.fail_next_alloc = false;
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("level %d buffer of %llu nodes (%llu bytes) failed: %s", L, (unsigned long long)cap,
                  (unsigned long long)bytes, cudaGetErrorString(e));
        return PG_ERR_OUT_OF_MEMORY;
    }
    unsigned char* p = (unsigned char*)blk;
    lb.v.pl0 = (ulonglong2*)p;
    p += cap * 16;
    lb.v.pl1 = (ulonglong2*)p;
    p += cap * 16;
    lb.v.pl2 = (ulonglong2*)p;
    p += cap * 16;
    lb.offs = (u64*)p;
    p += (cap + 1) * 8;
    p = (unsigned char*)(((uintptr_t)p + 15) & ~(uintptr_t)15);
    lb.v.grp = (u32*)p;
    p += cap * 4;
    lb.cnt = (u32*)p;
    p += cap * 4;
    lb.v.rem = p;
    lb.cap = cap;
    lb.block = blk;
    E.level_bytes_total += cap * NODE_BYTES;
    return PG_OK;
}

// ---------------------------------------------------------------------------
// breadth-first driver
// ---------------------------------------------------------------------------

// the leaf kernel's variant at level L: nodes finishing there come from roots
// of depth L + leaf_plies, and the tuner picked a variant per root depth
static Variant leaf_variant(const Variant& v, int L)
{
    Engine& E = engine();
    if (!v.per_depth || !E.tuned) return v;
    Variant w = v;
    const int d = std::min(L + v.leaf_plies, 15);
    if (E.tuned_slider[d]) {
        w.slider = E.tuned_slider[d];
        w.T = E.tuned_T[d];
    }
    return w;
}

// adds the leaf launches timed since the last call to the stats; every
// recorded event must be complete (the caller synchronised the stream)
static void collect_leaf_timers()
{
    Engine& E = engine();
    for (size_t i = 0; i + 1 < E.leaf_ev_used; i += 2) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, E.leaf_ev[i], E.leaf_ev[i + 1]) == cudaSuccess)
            E.st.leaf_kernel_ms += ms;
        else
            (void)cudaGetLastError();  // a pair left unrecorded by a failed call: no stale error
    }
    E.leaf_ev_used = 0;
}

// an event pair for the next leaf launch (created on first use, kept)
static int leaf_timer_pair(cudaEvent_t*& pair)
{
    Engine& E = engine();
    if (E.leaf_ev_used >= 512) {  // bound the pool: wait for the recorded ones
        PG_CUDA(cudaEventSynchronize(E.leaf_ev[E.leaf_ev_used - 1]));
        collect_leaf_timers();
    }
    while (E.leaf_ev.size() < E.leaf_ev_used + 2) {
        cudaEvent_t ev;
        PG_CUDA(cudaEventCreate(&ev));
        E.leaf_ev.push_back(ev);
    }
    pair = &E.leaf_ev[E.leaf_ev_used];
    E.leaf_ev_used += 2;
    return PG_OK;
}

static int run_range(const Variant& v, int L, u32 start, u32 n, int side, int minrem, int maxrem, u64* acc)
{
    Engine& E = engine();
    if (n == 0) return PG_OK;
    LevelBuf& lb = E.lv[L];
    E.st.peak_level_bytes = std::max<uint64_t>(E.st.peak_level_bytes, (uint64_t)n * 48);
    const int lp = v.leaf_plies;
    const bool capturing = E.plan_mode == PLAN_REPLAY;
    if (minrem <= lp) {
        cudaEvent_t* ev = nullptr;
        if (!capturing) {
            PG_TRY(leaf_timer_pair(ev));
            cudaEventRecord(ev[0], E.stream);
        }
        PG_TRY(launch_leaf(leaf_variant(v, L), side, lb.v, start, n, acc));
        if (!capturing) cudaEventRecord(ev[1], E.stream);
    }
    if (maxrem <= lp) return PG_OK;
    PG_TRY(launch_count(v, side, lb.v, start, n, lb.cnt));
    PG_TRY(launch_scan(lb.cnt, n, lb.offs));
    std::vector<u32> bnd;
    std::vector<u64> boff;
    if (capturing) {
        // the chunk plan recorded by the previous run of the same inputs
        if (E.rec_next >= E.rec_bnd.size()) {
            set_error("recorded launch plan does not match the inputs");
            return PG_ERR_INVALID_ARGUMENT;
        }
        bnd = E.rec_bnd[E.rec_next];
        boff = E.rec_off[E.rec_next];
        E.rec_next++;
    } else {
        const u64 cap_next = level_cap_max();
        k_plan<<<1, 32, 0, E.stream>>>(lb.offs, n, cap_next, E.plan_dev, E.err);
        PG_CUDA(cudaGetLastError());
        E.st.launches++;
        u32* perr = (u32*)(E.host_scratch + 192);  // pinned
        PG_CUDA(cudaMemcpyAsync(E.plan_host, E.plan_dev, sizeof(PlanOut), cudaMemcpyDeviceToHost, E.stream));
        PG_CUDA(cudaMemcpyAsync(perr, E.err, sizeof(u32), cudaMemcpyDeviceToHost, E.stream));
        PG_CUDA(cudaStreamSynchronize(E.stream));
        collect_leaf_timers();
        const u32 errv = *perr;
        if (errv) {
            set_error("device error flags 0x%x while planning level %d", errv, L);
            return PG_ERR_DEVICE_TIMEOUT;
        }
        const PlanOut& plan = *E.plan_host;  // copied out: deeper levels reuse the pinned buffer
        bnd.assign(plan.bnd, plan.bnd + plan.nchunks + 1);
        boff.assign(plan.coff, plan.coff + plan.nchunks + 1);
        if (E.plan_mode == PLAN_RECORD) {
            E.rec_bnd.push_back(bnd);
            E.rec_off.push_back(boff);
        }
    }
    if (boff.back() == boff.front()) return PG_OK;
    const int cminrem = std::max(minrem, lp + 1) - 1, cmaxrem = maxrem - 1;
    for (size_t k = 0; k + 1 < bnd.size(); k++) {
        const u32 a = bnd[k], b = bnd[k + 1];
        const u64 children = boff[k + 1] - boff[k];
        if (!children) continue;
        PG_TRY(ensure_level(L + 1, children));
        PG_TRY(launch_expand(v, side, lb.v, start, a, b, lb.offs, E.lv[L + 1].v));
        PG_TRY(run_range(v, L + 1, 0, (u32)children, 1 - side, cminrem, cmaxrem, acc));
    }
    return PG_OK;
}

// The autotuner: per root depth 3..6, a seeded calibration batch is timed
// with each candidate leaf variant (slider policy x CTA size); the fastest
// serves that depth (shallower depths take depth 3's, deeper ones depth 6's).
// The switch depth (last one or two plies inside the CTA) is chosen on the
// depth-5 batch.  Runs once per engine, on the first call that leaves the
// choice to it; its own buffers, so a caller's staged inputs are untouched.
static int autotune_locked()
{
    Engine& E = engine();
    if (E.tuned) return PG_OK;
    const auto t0 = std::chrono::steady_clock::now();
    const pg_stats saved = E.st;
    struct Cal {
        int depth;
        u32 n;
    };
    const Cal cals[] = {{3, 2048}, {4, 512}, {5, 64}, {6, 4}};
    const int cand[][2] = {{PG_SLIDER_KOGGE_STONE, 128}, {PG_SLIDER_KOGGE_STONE, 256}, {PG_SLIDER_KOGGE_STONE, 512},
                           {PG_SLIDER_FANCY, 256},        {PG_SLIDER_FANCY, 512},        {PG_SLIDER_BYTE_SMEM, 512},
                           {PG_SLIDER_HYBRID, 256},       {PG_SLIDER_HYBRID, 512}};
    const int ncand = (int)(sizeof(cand) / sizeof(cand[0]));
    const u32 nmax = 2048;
    void* buf = nullptr;
    PG_CUDA(cudaMalloc(&buf, nmax * (48 + 1 + 8) + 256));
    Pos* d_pos = (Pos*)buf;
    unsigned char* d_dep = (unsigned char*)buf + nmax * 48;
    u64* d_out = (u64*)(((uintptr_t)(d_dep + nmax) + 15) & ~(uintptr_t)15);
    pg_board start;
    pg_board_from_fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1", &start);
    Pos sp;
    memcpy(&sp, &start, sizeof(sp));
    int rc = PG_OK;
    auto time_run = [&](const Cal& c, const Variant& v, double& best) {
        for (int rep = 0; rep < 2 && rc == PG_OK; rep++) {
            rc = perft_core(d_pos, d_dep, nullptr, c.n, d_out, true, v);
            if (rc == PG_OK && E.st.device_ms > 0) best = std::min(best, E.st.device_ms);
        }
    };
    for (const Cal& c : cals) {
        if (rc != PG_OK) break;
        cudaError_t e = g_ops_ks.playouts(sp, 0x7E57ull + c.depth, c.n, 0, 60, 1, c.depth, c.depth, d_pos, d_dep,
                                          E.err, E.stream);
        if (e != cudaSuccess) {
            rc = PG_ERR_CUDA;
            break;
        }
        double best_ms = 1e30;
        int best = 1;
        for (int k = 0; k < ncand && rc == PG_OK; k++) {
            Variant v;
            v.slider = cand[k][0];
            v.T = cand[k][1];
            double ms = 1e30;
            time_run(c, v, ms);
            if (ms < best_ms) {
                best_ms = ms;
                best = k;
            }
        }
        u64 leaves = 0;
        std::vector<u64> out(c.n);
        if (rc == PG_OK && cudaMemcpy(out.data(), d_out, c.n * 8, cudaMemcpyDeviceToHost) == cudaSuccess)
            for (u64 x : out) leaves += x;
        E.tuned_slider[c.depth] = cand[best][0];
        E.tuned_T[c.depth] = cand[best][1];
        E.tuned_rate[c.depth] = best_ms < 1e29 ? leaves / (best_ms * 1e-3) : 0;
        if (c.depth == 5 && rc == PG_OK) {  // switch depth on the depth-5 batch
            Variant v;
            v.slider = cand[best][0];
            v.T = cand[best][1];
            v.leaf_plies = 1;
            double ms1 = 1e30;
            time_run(c, v, ms1);
            E.tuned_leaf_plies = ms1 < best_ms ? 1 : 2;
        }
    }
    cudaFree(buf);
    if (rc != PG_OK) return rc;
    for (int d = 0; d < 3; d++) {
        E.tuned_slider[d] = E.tuned_slider[3];
        E.tuned_T[d] = E.tuned_T[3];
    }
    for (int d = 7; d < 16; d++) {
        E.tuned_slider[d] = E.tuned_slider[6];
        E.tuned_T[d] = E.tuned_T[6];
    }
    E.st = saved;
    E.tuned = true;
    E.tune_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return PG_OK;
}

// resolves the options to a launch variant; slider, block size and switch
// depth left at 0 (auto) come from the autotuner, which runs on first use
Variant pick_variant(const pg_opts* o)
{
    Engine& E = engine();
    Variant v;
    int sl = o ? o->slider : PG_SLIDER_AUTO;
    if (sl == PG_SLIDER_AUTO) sl = E.default_slider;
    const bool auto_all = sl == PG_SLIDER_AUTO && !(o && o->block_size) && !(o && o->leaf_plies);
    if (auto_all && !E.tuned) autotune_locked();
    if (auto_all && E.tuned) {
        v.per_depth = true;
        v.leaf_plies = E.tuned_leaf_plies;
        v.slider = PG_SLIDER_KOGGE_STONE;  // expansions; leaves use the table
        return v;
    }
    v.slider = sl == PG_SLIDER_AUTO ? PG_SLIDER_KOGGE_STONE : sl;
    if (o && (o->block_size == 128 || o->block_size == 256 || o->block_size == 512)) v.T = o->block_size;
    if (o && (o->leaf_plies == 1 || o->leaf_plies == 2)) v.leaf_plies = o->leaf_plies;
    return v;
}

static bool valid_board(const pg_board& b)
{
    const u64 inner = INNER;
    const u64 pawns = b.pawns & inner;
    const u64 occ = pawns | b.knights | b.bishop_queens | b.rook_queens | b.kings;
    if (pawns & (b.knights | b.bishop_queens | b.rook_queens | b.kings)) return false;
    if (b.knights & (b.bishop_queens | b.rook_queens | b.kings)) return false;
    if ((b.bishop_queens | b.rook_queens) & b.kings) return false;
    if (b.white & ~occ) return false;
    if (__builtin_popcountll(b.kings & b.white) != 1) return false;
    if (__builtin_popcountll(b.kings & ~b.white) != 1) return false;
    return true;
}

static int check_opts(const pg_opts* o)
{
    if (o && (o->use_tt < PG_TT_OFF || o->use_tt > PG_TT_DEDUP_ONLY)) {
        set_error("use_tt %d is not a pg_tt_mode", o->use_tt);
        return PG_ERR_INVALID_ARGUMENT;
    }
    return PG_OK;
}

static int check_ready()
{
    if (!engine().ready) {
        set_error("pg_init has not been called");
        return PG_ERR_NOT_INITIALIZED;
    }
    return PG_OK;
}

int ensure_stage(u64 bytes)
{
    Engine& E = engine();
    if (E.stage_cap >= bytes) return PG_OK;
    E.alloc_gen++;
    if (E.stage) cudaFree(E.stage);
    E.stage = nullptr;
    E.stage_cap = 0;
    u64 cap = 1 << 20;
    while (cap < bytes) cap <<= 1;
    PG_CUDA(cudaMalloc(&E.stage, cap));
    E.stage_cap = cap;
    return PG_OK;
}

static int begin_call(const pg_opts* o)
{
    Engine& E = engine();
    E.st = pg_stats{};
    E.leaf_ev_used = 0;
    E.ticket_next = 0;
    PG_CUDA(cudaMemsetAsync(E.tickets, 0, MAX_TICKETS * sizeof(u32), E.stream));
    PG_CUDA(cudaMemsetAsync(E.err, 0, sizeof(u32), E.stream));
    (void)o;
    return PG_OK;
}

static int end_call(const pg_opts* o)
{
    Engine& E = engine();
    u32 errv = 0;
    PG_CUDA(cudaMemcpyAsync(E.host_scratch, E.err, sizeof(u32), cudaMemcpyDeviceToHost, E.stream));
    PG_CUDA(cudaStreamSynchronize(E.stream));
    errv = (u32)E.host_scratch[0];
    if (errv & (ERR_PLAN_OVERFLOW | ERR_LEVEL_CAP)) {
        set_error("device error flags 0x%x: the work exceeded a fixed-size plan or level", errv);
        return PG_ERR_CAPACITY;
    }
    if (errv & 0xFFFFFFFFu) {
        set_error("device error flags 0x%x", errv);
        return PG_ERR_DEVICE_TIMEOUT;
    }
    if (o && o->stats) *o->stats = E.st;
    return PG_OK;
}

// perft of n roots; each root's count is added to acc[group] (group =
// groups[i], or i when groups is null).  acc is zeroed first when zero_acc.
int perft_core(const Pos* d_pos, const unsigned char* d_depths, const u32* d_groups, u32 n, u64* acc, bool zero_acc,
               const Variant& v)
{
    Engine& E = engine();
    const bool capturing = E.plan_mode == PLAN_REPLAY;
    E.leaf_ev_used = 0;
    PG_TRY(ensure_level(0, n));
    if (zero_acc) PG_CUDA(cudaMemsetAsync(acc, 0, (u64)n * sizeof(u64), E.stream));
    u32* ctr = (u32*)(E.host_scratch + 64);  // pinned, 4 words
    u32* dctr = E.tickets + MAX_TICKETS - 4;  // white count, black count, min depth, max depth
    PG_CUDA(cudaMemsetAsync(dctr, 0, 4 * sizeof(u32), E.stream));
    PG_CUDA(cudaMemsetAsync(dctr + 2, 0xFF, sizeof(u32), E.stream));
    k_partition_roots<<<std::max<u32>(1, std::min<u32>((n + 255) / 256, 4096)), 256, 0, E.stream>>>(
        d_pos, d_depths, n, E.lv[0].v, dctr, d_groups);
    PG_CUDA(cudaGetLastError());
    E.st.launches++;
    u32 nw, mind, maxd;
    if (capturing) {
        nw = E.rec_part[0];
        mind = E.rec_part[2];
        maxd = E.rec_part[3];
    } else {
        PG_CUDA(cudaMemcpyAsync(ctr, dctr, 4 * sizeof(u32), cudaMemcpyDeviceToHost, E.stream));
        PG_CUDA(cudaStreamSynchronize(E.stream));
        nw = ctr[0];
        mind = ctr[2];
        maxd = ctr[3];
        if (E.plan_mode == PLAN_RECORD) memcpy(E.rec_part, ctr, sizeof(E.rec_part));
    }
    if (maxd > 15) {
        set_error("depth %u out of range 0..15", maxd);
        return PG_ERR_INVALID_ARGUMENT;
    }
    if (!capturing) cudaEventRecord(E.ev0, E.stream);
    PG_TRY(run_range(v, 0, 0, nw, 0, (int)mind, (int)maxd, acc));
    PG_TRY(run_range(v, 0, nw, n - nw, 1, (int)mind, (int)maxd, acc));
    if (!capturing) {
        cudaEventRecord(E.ev1, E.stream);
        PG_CUDA(cudaEventSynchronize(E.ev1));
        float ms = 0;
        cudaEventElapsedTime(&ms, E.ev0, E.ev1);
        E.st.device_ms = ms;
        collect_leaf_timers();
    }
    return PG_OK;
}

int perft_core_persistent(const Pos* d_pos, const unsigned char* d_depths, const u32* d_groups, u32 n, u64* acc,
                          bool zero_acc, int maxd);
static int prepare_persist(u32 n, int maxd, PersistArgs& A);
static int device_max_depth(const unsigned char* d_depths, u32 n, int* maxd);

// The persistent launch replayed from a graph: its chunk plans are made on
// the device, so a captured graph (a few memsets and the one cooperative
// launch) stays valid for any contents of the same buffers, size and largest
// depth (the level buffers are prepared for it); only the largest depth is
// read back per call.
static int perft_batch_graph_persistent(const Pos* d_pos, const unsigned char* d_depths, u32 n, u64* d_out)
{
    Engine& E = engine();
    int maxd = 0;
    PG_TRY(device_max_depth(d_depths, n, &maxd));
    if (maxd > 15) {
        set_error("depth %d out of range 0..15", maxd);
        return PG_ERR_INVALID_ARGUMENT;
    }
    GraphCache& g = E.graph;
    const bool hit = g.exec && g.persistent && g.alloc_gen == E.alloc_gen && g.pos == d_pos && g.dep == d_depths &&
                     g.out == d_out && g.n == n && g.maxd == maxd;
    if (!hit) {
        PersistArgs A;
        PG_TRY(prepare_persist(n, maxd, A));  // every allocation before the capture
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = GraphCache{};
        cudaGraph_t graph = nullptr;
        PG_CUDA(cudaStreamBeginCapture(E.stream, cudaStreamCaptureModeThreadLocal));
        E.plan_mode = PLAN_REPLAY;
        const int rc = perft_core_persistent(d_pos, d_depths, nullptr, n, d_out, true, maxd);
        E.plan_mode = PLAN_NONE;
        const cudaError_t ce = cudaStreamEndCapture(E.stream, &graph);
        if (rc != PG_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        PG_CUDA(ce);
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        PG_CUDA(ie);
        g.exec = exec;
        g.persistent = true;
        g.maxd = maxd;
        g.pos = d_pos;
        g.dep = d_depths;
        g.out = d_out;
        g.n = n;
        g.launches = 1;
        g.alloc_gen = E.alloc_gen;
        E.st.graph_captures = 1;
    } else {
        E.st.graph_replays = 1;
    }
    cudaEventRecord(E.ev0, E.stream);
    PG_CUDA(cudaGraphLaunch(g.exec, E.stream));
    cudaEventRecord(E.ev1, E.stream);
    PG_CUDA(cudaEventSynchronize(E.ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, E.ev0, E.ev1);
    E.st.device_ms = ms;
    E.st.leaf_kernel_ms = ms;
    E.st.launches = 1;
    return PG_OK;
}

// Batch perft replayed from a captured CUDA graph.  The first call on a set
// of inputs runs normally while recording its data-dependent launch plan
// (root partition, chunk boundaries), then captures the same launch sequence
// without any host synchronisation into a graph; later calls whose inputs
// (pointers, size, and a device checksum of the contents) and variant are
// unchanged launch that graph.
static int perft_batch_graph_locked(const Pos* d_pos, const unsigned char* d_depths, u32 n, u64* d_out,
                                    const pg_opts* o)
{
    Engine& E = engine();
    const Variant v = pick_variant(o);
    PG_CUDA(cudaMemsetAsync(E.aux, 0, sizeof(u64), E.stream));
    k_checksum<<<std::max<u32>(1, std::min<u32>((n + 255) / 256, 1024)), 256, 0, E.stream>>>(d_pos, d_depths, n,
                                                                                           E.aux);
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaMemcpyAsync(E.host_scratch + 128, E.aux, sizeof(u64), cudaMemcpyDeviceToHost, E.stream));
    PG_CUDA(cudaStreamSynchronize(E.stream));
    const u64 sum = E.host_scratch[128];
    GraphCache& g = E.graph;
    // a graph names the level, scan and staging buffers of its capture: any
    // reallocation since (alloc_gen) makes it stale, never replayed
    const bool hit = g.exec && !g.persistent && g.alloc_gen == E.alloc_gen && g.pos == d_pos && g.dep == d_depths && g.out == d_out &&
                     g.n == n && g.sum == sum && g.slider == v.slider && g.T == v.T &&
                     g.leaf_plies == v.leaf_plies && g.per_depth == v.per_depth;
    if (hit) {
        cudaEventRecord(E.ev0, E.stream);
        PG_CUDA(cudaGraphLaunch(g.exec, E.stream));
        cudaEventRecord(E.ev1, E.stream);
        PG_CUDA(cudaEventSynchronize(E.ev1));
        float ms = 0;
        cudaEventElapsedTime(&ms, E.ev0, E.ev1);
        E.st.device_ms = ms;
        E.st.launches = g.launches;
        E.st.graph_replays = 1;
        return PG_OK;
    }
    // record: a normal run computes this call's result and the launch plan
    E.rec_bnd.clear();
    E.rec_off.clear();
    E.plan_mode = PLAN_RECORD;
    int rc = perft_core(d_pos, d_depths, nullptr, n, d_out, true, v);
    E.plan_mode = PLAN_NONE;
    if (rc != PG_OK) return rc;
    const pg_stats rec_stats = E.st;
    // capture the same launches with the recorded plan
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = GraphCache{};
    const u32 tickets_used = E.ticket_next;
    E.ticket_next = 0;
    E.rec_next = 0;
    cudaGraph_t graph = nullptr;
    PG_CUDA(cudaStreamBeginCapture(E.stream, cudaStreamCaptureModeThreadLocal));
    E.plan_mode = PLAN_REPLAY;
    cudaMemsetAsync(E.tickets, 0, (u64)tickets_used * sizeof(u32), E.stream);
    cudaMemsetAsync(E.err, 0, sizeof(u32), E.stream);
    rc = perft_core(d_pos, d_depths, nullptr, n, d_out, true, v);
    E.plan_mode = PLAN_NONE;
    const cudaError_t ce = cudaStreamEndCapture(E.stream, &graph);
    E.st = rec_stats;
    if (rc != PG_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    PG_CUDA(ce);
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    PG_CUDA(ie);
    g.exec = exec;
    g.pos = d_pos;
    g.dep = d_depths;
    g.out = d_out;
    g.n = n;
    g.sum = sum;
    g.slider = v.slider;
    g.T = v.T;
    g.leaf_plies = v.leaf_plies;
    g.per_depth = v.per_depth;
    g.launches = rec_stats.launches;
    g.alloc_gen = E.alloc_gen;
    E.st.graph_captures = 1;
    return PG_OK;
}

// The buffers of a persistent launch of roots up to depth maxd: every level
// down to the leaf-parent level (maxd - 2, the two-ply leaf) is prepared
// before the launch.  The leaf-parent level gets up to the largest level
// (level_cap_max), each level above it a 16th of the one below (a chunk of
// it still fills the level below about twice), no level less than 65,536
// nodes or more than it can hold (n x 40^L): chunks keep the launch correct
// at any capacity.
static int prepare_persist(u32 n, int maxd, PersistArgs& A)
{
    Engine& E = engine();
    memset(&A, 0, sizeof(A));
    const int deepest = std::min(std::max(maxd - 2, 0), MAX_LEVELS - 1);
    const u64 capmax = level_cap_max();
    u64 status_words = 0;
    for (int L = 0; L <= deepest; L++) {
        u64 cap = n;
        if (L > 0) {
            double est = (double)n;
            for (int k = 0; k < L; k++) est *= 40.0;
            const u64 bound = capmax >> std::min(60, 4 * (deepest - L));
            cap = (u64)std::min(est, (double)bound);
            cap = std::max<u64>(cap, 1u << 16);
        }
        PG_TRY(ensure_level(L, cap));
        const LevelBuf& lb = E.lv[L];
        A.lv[L] = lb.v;
        A.cnt[L] = lb.cnt;
        A.offs[L] = lb.offs;
        A.cap[L] = lb.cap;
        status_words = std::max<u64>(status_words, lb.cap / PERSIST_SCAN_TILE_NODES + 2);
    }
    if (status_words > E.scan_status_cap) {
        E.alloc_gen++;
        PG_CUDA(cudaStreamSynchronize(E.stream));
        if (E.scan_status) cudaFree(E.scan_status);
        E.scan_status = nullptr;
        E.scan_status_cap = 0;
        PG_CUDA(cudaMalloc(&E.scan_status, status_words * sizeof(u64)));
        E.scan_status_cap = status_words;
    }
    if (!E.persist_plan) PG_CUDA(cudaMalloc(&E.persist_plan, MAX_LEVELS * sizeof(PlanOut)));
    if (!E.persist_ctl) PG_CUDA(cudaMalloc(&E.persist_ctl, sizeof(PersistCtl)));
    A.plan = E.persist_plan;
    A.status = E.scan_status;
    A.status_cap = E.scan_status_cap;
    A.tickets = E.tickets;
    A.max_tickets = MAX_TICKETS - 8;
    A.ctl = E.persist_ctl;
    A.err = E.err;
    return PG_OK;
}

// the largest depth of a device batch (one readback)
static int device_max_depth(const unsigned char* d_depths, u32 n, int* maxd)
{
    Engine& E = engine();
    u32* d = (u32*)E.aux;
    PG_CUDA(cudaMemsetAsync(d, 0, sizeof(u32), E.stream));
    k_max_depth<<<std::max<u32>(1, std::min<u32>((n + 255) / 256, 1024)), 256, 0, E.stream>>>(d_depths, n, d);
    PG_CUDA(cudaGetLastError());
    u32* h = (u32*)(E.host_scratch + 160);
    PG_CUDA(cudaMemcpyAsync(h, d, sizeof(u32), cudaMemcpyDeviceToHost, E.stream));
    PG_CUDA(cudaStreamSynchronize(E.stream));
    *maxd = (int)*h;
    return PG_OK;
}

// perft of n roots in one persistent launch; each root's count is added to
// acc[group] (group = groups[i], or i when groups is null), acc zeroed first
// when zero_acc; maxd = the largest depth of the roots
int perft_core_persistent(const Pos* d_pos, const unsigned char* d_depths, const u32* d_groups, u32 n, u64* acc,
                          bool zero_acc, int maxd)
{
    Engine& E = engine();
    if (maxd > 15) {
        set_error("depth %d out of range 0..15", maxd);
        return PG_ERR_INVALID_ARGUMENT;
    }
    PersistArgs A;
    PG_TRY(prepare_persist(n, maxd, A));
    A.pos = d_pos;
    A.depths = d_depths;
    A.groups = d_groups;
    A.n = n;
    A.acc = acc;
    if (zero_acc) PG_CUDA(cudaMemsetAsync(acc, 0, (u64)n * sizeof(u64), E.stream));
    PG_CUDA(cudaMemsetAsync(E.persist_ctl, 0, sizeof(PersistCtl), E.stream));
    PG_CUDA(cudaMemsetAsync(&E.persist_ctl->part[2], 0xFF, sizeof(u32), E.stream));
    PG_CUDA(cudaMemsetAsync(E.tickets, 0, MAX_TICKETS * sizeof(u32), E.stream));
    const bool capturing = E.plan_mode == PLAN_REPLAY;
    if (!capturing) cudaEventRecord(E.ev0, E.stream);
    int grid = 0;
    PG_CUDA(persist_launch(A, E.stream, E.num_sms, &grid));
    E.st.launches++;
    if (!capturing) {
        cudaEventRecord(E.ev1, E.stream);
        PG_CUDA(cudaEventSynchronize(E.ev1));
        float ms = 0;
        cudaEventElapsedTime(&ms, E.ev0, E.ev1);
        E.st.device_ms = ms;
        E.st.leaf_kernel_ms = ms;  // one kernel: its leaf phases are not timed apart
    }
    return PG_OK;
}

// batch perft with device inputs; d_out must not alias the inputs; maxd the
// batch's largest depth when the caller knows it (else -1)
static int perft_batch_device_locked(const Pos* d_pos, const unsigned char* d_depths, u32 n, u64* d_out,
                                     const pg_opts* o, int maxd = -1)
{
    if (o && o->persistent) {
        if (maxd < 0) PG_TRY(device_max_depth(d_depths, n, &maxd));
        return perft_core_persistent(d_pos, d_depths, nullptr, n, d_out, true, maxd);
    }
    return perft_core(d_pos, d_depths, nullptr, n, d_out, true, pick_variant(o));
}

// The positions `plies` plies below root (all of them, in generateMoves
// order level by level), written to out as boards; *n_out = their number.
// Fails with PG_ERR_CAPACITY when they exceed cap or one level buffer; *n_out
// is then the size of the level that did not fit (a lower bound of the
// space the frontier needs).
int expand_frontier(const Pos& root, int plies, Pos* out, u32 cap, u32* n_out)
{
    Engine& E = engine();
    const Variant v = pick_variant(nullptr);
    E.ticket_next = 0;
    PG_CUDA(cudaMemsetAsync(E.tickets, 0, MAX_TICKETS * sizeof(u32), E.stream));
    PG_CUDA(cudaMemsetAsync(E.err, 0, sizeof(u32), E.stream));
    PG_TRY(ensure_level(0, 1));
    PG_TRY(ensure_stage(64));
    Pos* d_root = (Pos*)E.stage;
    unsigned char* d_dep = (unsigned char*)E.stage + 48;
    const unsigned char rem = (unsigned char)(plies + 3);  // >= 3 at every level that is expanded
    PG_CUDA(cudaMemcpyAsync(d_root, &root, sizeof(Pos), cudaMemcpyHostToDevice, E.stream));
    PG_CUDA(cudaMemcpyAsync(d_dep, &rem, 1, cudaMemcpyHostToDevice, E.stream));
    u32* dctr = E.tickets + MAX_TICKETS - 4;
    const u32 init[4] = {0, 0, 0xFFFFFFFFu, 0};
    PG_CUDA(cudaMemcpyAsync(dctr, init, sizeof(init), cudaMemcpyHostToDevice, E.stream));
    k_partition_roots<<<1, 32, 0, E.stream>>>(d_root, d_dep, 1, E.lv[0].v, dctr, nullptr);
    PG_CUDA(cudaGetLastError());
    int side = (int)(root.p >> 63);
    u32 n = 1;
    for (int L = 0; L < plies; L++) {
        LevelBuf& lb = E.lv[L];
        PG_TRY(launch_count(v, side, lb.v, 0, n, lb.cnt));
        PG_TRY(launch_scan(lb.cnt, n, lb.offs));
        u64 total = 0;
        PG_CUDA(cudaMemcpyAsync(E.host_scratch, lb.offs + n, sizeof(u64), cudaMemcpyDeviceToHost, E.stream));
        PG_CUDA(cudaStreamSynchronize(E.stream));
        total = E.host_scratch[0];
        if (total > cap || total > level_cap_max()) {
            set_error("frontier of %llu positions exceeds the capacity %u", (unsigned long long)total, cap);
            *n_out = (u32)std::min<u64>(total, 0xFFFFFFFFull);  // a lower bound of the space needed
            return PG_ERR_CAPACITY;
        }
        if (total == 0) {
            n = 0;
            break;
        }
        PG_TRY(ensure_level(L + 1, total));
        PG_TRY(launch_expand(v, side, lb.v, 0, 0, n, lb.offs, E.lv[L + 1].v));
        n = (u32)total;
        side ^= 1;
    }
    if (n) {
        k_level_to_boards<<<std::max<u32>(1, std::min<u32>((n + 255) / 256, 4096)), 256, 0, E.stream>>>(
            E.lv[plies].v, n, out);
        PG_CUDA(cudaGetLastError());
    }
    PG_CUDA(cudaStreamSynchronize(E.stream));
    *n_out = n;
    return PG_OK;
}

// ---------------------------------------------------------------------------
// divided perft at deep roots with a host-side complete transposition table
// ---------------------------------------------------------------------------

struct BoardKey {
    u64 w[6];
    bool operator==(const BoardKey& o) const { return !memcmp(w, o.w, sizeof(w)); }
};
struct BoardKeyHash {
    size_t operator()(const BoardKey& k) const
    {
        u64 h = 0xCBF29CE484222325ull;
        for (u64 x : k.w) {
            h ^= x;
            h *= 0x100000001B3ull;
            h ^= h >> 29;
        }
        return (size_t)h;
    }
};

// perft_bb_cpu_launcher (launcher.h:1181-1389) re-planned: every root move's
// positions split_plies below the root are made on the GPU, merged across all
// root moves in a host table keyed by the full board (the reference's
// complete TT, launcher.h:598-680, without its hash collisions), and each
// distinct position is counted once, in one batched engine call.
int perft_split_locked(const Pos& root, int depth, int split, u16* moves, u64* counts, u32* nmoves,
                       const pg_opts* o)
{
    Engine& E = engine();
    if (split < 1) split = 1;
    if (split > depth) split = depth;
    // root moves and children (generateMoves order, makeMove children)
    PG_TRY(ensure_stage(256 * 48 + 512 + 64));
    Pos* d = (Pos*)E.stage;
    u16* dm = (u16*)((unsigned char*)E.stage + 256 * 48);
    u32* dn = (u32*)((unsigned char*)E.stage + 256 * 48 + 512);
    PG_CUDA(cudaMemcpyAsync(d, &root, sizeof(Pos), cudaMemcpyHostToDevice, E.stream));
    PG_CUDA(g_ops_ks.gen_moves_batch(d, 1, dm, dn, E.stream));
    u32 n = 0;
    PG_CUDA(cudaMemcpyAsync(moves, dm, 512, cudaMemcpyDeviceToHost, E.stream));
    PG_CUDA(cudaMemcpyAsync(&n, dn, 4, cudaMemcpyDeviceToHost, E.stream));
    PG_CUDA(cudaStreamSynchronize(E.stream));
    if (n > 256) {
        set_error("more than 256 moves");
        return PG_ERR_CAPACITY;
    }
    *nmoves = n;
    if (!n) return PG_OK;
    std::vector<Pos> kids(n, root);
    PG_CUDA(cudaMemcpyAsync(d, kids.data(), n * sizeof(Pos), cudaMemcpyHostToDevice, E.stream));
    PG_CUDA(g_ops_ks.make_batch(d, dm, n, E.stream));
    PG_CUDA(cudaMemcpyAsync(kids.data(), d, n * sizeof(Pos), cudaMemcpyDeviceToHost, E.stream));
    PG_CUDA(cudaStreamSynchronize(E.stream));
    const int rest = depth - split;  // depth left under each split position
    std::unordered_map<BoardKey, u32, BoardKeyHash> table;
    std::vector<Pos> uniq;
    std::vector<std::vector<std::pair<u32, u64>>> uses(n);  // (unique index, multiplicity) per root move
    const u32 cap = 1u << 24;
    Pos* frontier = nullptr;
    PG_CUDA(cudaMalloc(&frontier, (u64)cap * sizeof(Pos)));
    std::vector<Pos> host;
    int rc = PG_OK;
    for (u32 i = 0; i < n && rc == PG_OK; i++) {
        u32 m = 0;
        if (split == 1) {
            host.assign(1, kids[i]);
            m = 1;
        } else {
            rc = expand_frontier(kids[i], split - 1, frontier, cap, &m);
            if (rc != PG_OK) break;
            host.resize(m);
            if (m && cudaMemcpy(host.data(), frontier, (u64)m * sizeof(Pos), cudaMemcpyDeviceToHost) != cudaSuccess)
                rc = PG_ERR_CUDA;
        }
        std::unordered_map<u32, u64> mult;
        for (u32 k = 0; k < m; k++) {
            BoardKey key;
            memcpy(key.w, &host[k], sizeof(key.w));
            key.w[1] &= ~(0x7Full << 56);  // the half-move clock does not change the count
            auto it = table.find(key);
            u32 u;
            if (it == table.end()) {
                u = (u32)uniq.size();
                table.emplace(key, u);
                uniq.push_back(host[k]);
            } else {
                u = it->second;
            }
            mult[u]++;
        }
        uses[i].assign(mult.begin(), mult.end());
    }
    cudaFree(frontier);
    if (rc != PG_OK) return rc;
    // count every distinct split position once
    const u32 U = (u32)uniq.size();
    std::vector<u64> res(U, 0);
    if (U) {
        PG_TRY(ensure_stage((u64)U * (48 + 1 + 8) + 64));
        Pos* dp = (Pos*)E.stage;
        unsigned char* dd = (unsigned char*)E.stage + (u64)U * 48;
        u64* dout = (u64*)(((uintptr_t)(dd + U) + 15) & ~(uintptr_t)15);
        PG_CUDA(cudaMemcpyAsync(dp, uniq.data(), (u64)U * 48, cudaMemcpyHostToDevice, E.stream));
        PG_CUDA(cudaMemsetAsync(dd, rest, U, E.stream));
        if (o && o->use_tt) PG_TRY(tt_perft_batch_device(dp, dd, U, dout, o));
        else PG_TRY(perft_core(dp, dd, nullptr, U, dout, true, pick_variant(o)));
        PG_CUDA(cudaMemcpyAsync(res.data(), dout, (u64)U * 8, cudaMemcpyDeviceToHost, E.stream));
        PG_CUDA(cudaStreamSynchronize(E.stream));
    }
    u64 total_split = 0;
    for (u32 i = 0; i < n; i++) {
        u64 c = 0;
        for (auto& [u, k] : uses[i]) {
            c += k * res[u];
            total_split += k;
        }
        counts[i] = c;
    }
    E.st.leaves = 0;
    for (u32 i = 0; i < n; i++) E.st.leaves += counts[i];
    E.st.tt_probes += total_split;        // split positions looked up in the host table
    E.st.tt_hits += total_split - U;      // ... of which already present
    return PG_OK;
}

// bounded-wait self test: a scan tile whose predecessor never publishes gives
// up after its poll limit and raises the error bit (no fault, no hang)
int selftest_bounded_wait()
{
    Engine& E = engine();
    PG_TRY(ensure_stage(4096));
    u32* cnt = (u32*)E.stage;
    u64* offs = (u64*)((unsigned char*)E.stage + 1024);
    u64* status = (u64*)((unsigned char*)E.stage + 2048);
    u32* ticket = (u32*)((unsigned char*)E.stage + 3072);
    PG_CUDA(cudaMemsetAsync(E.stage, 0, 4096, E.stream));
    PG_CUDA(cudaMemsetAsync(E.err, 0, 4, E.stream));
    const u32 one = 1;  // the only block takes tile 1 and waits on tile 0, which no block runs
    PG_CUDA(cudaMemcpyAsync(ticket, &one, 4, cudaMemcpyHostToDevice, E.stream));
    k_scan<<<1, SCAN_T, 0, E.stream>>>(cnt, 4096, offs, status, ticket, E.err);
    PG_CUDA(cudaGetLastError());
    u32 err = 0;
    PG_CUDA(cudaMemcpyAsync(&err, E.err, 4, cudaMemcpyDeviceToHost, E.stream));
    PG_CUDA(cudaStreamSynchronize(E.stream));
    if (err & ERR_SCAN_TIMEOUT) {
        set_error("bounded wait gave up as designed (error bits 0x%x)", err);
        return PG_ERR_DEVICE_TIMEOUT;
    }
    set_error("bounded wait did not report its timeout");
    return PG_ERR_CUDA;
}

}  // namespace pg

using namespace pg;

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

const char* pg_last_error(void) { return t_error.c_str(); }

int pg_get_stream(void** stream)
{
    if (!stream) {
        set_error("null argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    PG_TRY(check_ready());
    *stream = (void*)engine().stream;
    return PG_OK;
}

// every resource the engine holds; handles that were never made are null
static void release_engine(Engine& E)
{
    if (E.stream) cudaStreamSynchronize(E.stream);
    for (auto& lb : E.lv) {
        if (lb.block) cudaFree(lb.block);
        lb = LevelBuf{};
    }
    tt_free();
    if (E.scan_status) cudaFree(E.scan_status);
    if (E.stage) cudaFree(E.stage);
    if (E.tickets) cudaFree(E.tickets);
    if (E.err) cudaFree(E.err);
    if (E.plan_dev) cudaFree(E.plan_dev);
    if (E.plan_host) cudaFreeHost(E.plan_host);
    if (E.host_scratch) cudaFreeHost(E.host_scratch);
    if (E.aux) cudaFree(E.aux);
    if (E.persist_plan) cudaFree(E.persist_plan);
    if (E.persist_ctl) cudaFree(E.persist_ctl);
    E.persist_plan = nullptr;
    E.persist_ctl = nullptr;
    if (E.graph.exec) cudaGraphExecDestroy(E.graph.exec);
    E.graph = GraphCache{};
    for (cudaEvent_t* ev : {&E.ev0, &E.ev1})
        if (*ev) cudaEventDestroy(*ev), *ev = nullptr;
    for (cudaEvent_t ev : E.leaf_ev) cudaEventDestroy(ev);
    E.leaf_ev.clear();
    E.leaf_ev_used = 0;
    if (E.stream) cudaStreamDestroy(E.stream);
    E.stream = nullptr;
    E.tickets = nullptr;
    E.err = nullptr;
    E.plan_dev = nullptr;
    E.plan_host = nullptr;
    E.host_scratch = nullptr;
    E.aux = nullptr;
    E.scan_status = nullptr;
    E.scan_status_cap = 0;
    E.stage = nullptr;
    E.stage_cap = 0;
    E.level_bytes_total = 0;
    E.ready = false;
}

static int init_locked(Engine& E, const pg_config* cfg)
{
    E.device = cfg ? cfg->device : 0;
    E.verbose = cfg ? cfg->verbose : 0;
    E.default_slider = cfg ? cfg->slider : PG_SLIDER_AUTO;
    int ndev = 0;
    PG_CUDA(cudaGetDeviceCount(&ndev));
    if (E.device < 0 || E.device >= ndev) {
        set_error("device %d not present (%d devices)", E.device, ndev);
        return PG_ERR_INVALID_ARGUMENT;
    }
    PG_CUDA(cudaSetDevice(E.device));
    cudaDeviceProp prop;
    PG_CUDA(cudaGetDeviceProperties(&prop, E.device));
    if (prop.major < 10) {
        set_error("device %d is sm_%d%d; this build targets sm_103a", E.device, prop.major, prop.minor);
        return PG_ERR_CUDA;
    }
    E.num_sms = prop.multiProcessorCount;
    size_t freeb = 0, totalb = 0;
    PG_CUDA(cudaMemGetInfo(&freeb, &totalb));
    E.budget = (cfg && cfg->hbm_budget_bytes) ? cfg->hbm_budget_bytes : (u64)(freeb * 0.6);
    PG_CUDA(cudaStreamCreateWithFlags(&E.stream, cudaStreamNonBlocking));
    PG_CUDA(cudaEventCreate(&E.ev0));
    PG_CUDA(cudaEventCreate(&E.ev1));
    const HostTables* tabs = host_tables();
    if (!tabs) {
        set_error("magic table construction failed");
        return PG_ERR_CUDA;
    }
    PG_CUDA(g_ops_ks.upload(*tabs));
    PG_CUDA(g_ops_fancy.upload(*tabs));
    PG_CUDA(g_ops_byte.upload(*tabs));
    PG_CUDA(g_ops_hybrid.upload(*tabs));
    PG_CUDA(cudaMalloc(&E.tickets, MAX_TICKETS * sizeof(u32)));
    PG_CUDA(cudaMalloc(&E.err, 16));
    PG_CUDA(cudaMalloc(&E.plan_dev, sizeof(PlanOut)));
    PG_CUDA(cudaMallocHost(&E.plan_host, sizeof(PlanOut)));
    PG_CUDA(cudaMallocHost(&E.host_scratch, 4096));
    PG_CUDA(cudaMalloc(&E.aux, 256));
    PG_CUDA(cudaDeviceSynchronize());
    E.ready = true;
    return PG_OK;
}

int pg_init(const pg_config* cfg)
{
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    if (E.ready) return PG_OK;
    const int rc = init_locked(E, cfg);
    if (rc != PG_OK) release_engine(E);  // a later pg_init starts clean
    return rc;
}

int pg_shutdown(void)
{
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    if (!E.ready) return PG_OK;
    release_engine(E);
    return PG_OK;
}

static int op_batch(int op, const pg_board* pos, u32 n, void* out, u32* nout, int slider)
{
    Engine& E = engine();
    const u64 in_bytes = (u64)n * sizeof(Pos);
    const u64 out_bytes = op == 0 ? (u64)n * 4 : op == 1 ? (u64)n * 512 : (u64)n * 256 * sizeof(Pos);
    const u64 nbytes = (u64)n * 4;
    PG_TRY(ensure_stage(in_bytes + out_bytes + nbytes + 64));
    unsigned char* s = (unsigned char*)E.stage;
    Pos* d_in = (Pos*)s;
    void* d_out = s + in_bytes;
    u32* d_n = (u32*)(s + in_bytes + out_bytes);
    PG_CUDA(cudaMemcpyAsync(d_in, pos, in_bytes, cudaMemcpyHostToDevice, E.stream));
    const SliderOps& ops = ops_for(slider);
    if (op == 0) PG_CUDA(ops.count_batch(d_in, n, (u32*)d_out, E.stream));
    else if (op == 1) PG_CUDA(ops.gen_moves_batch(d_in, n, (u16*)d_out, d_n, E.stream));
    else PG_CUDA(ops.gen_boards_batch(d_in, n, (Pos*)d_out, d_n, E.stream));
    PG_CUDA(cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, E.stream));
    if (nout) PG_CUDA(cudaMemcpyAsync(nout, d_n, nbytes, cudaMemcpyDeviceToHost, E.stream));
    PG_CUDA(cudaStreamSynchronize(E.stream));
    return PG_OK;
}

static int slider_of(int s)
{
    if (s == PG_SLIDER_AUTO) s = engine().default_slider;
    return s == PG_SLIDER_AUTO ? PG_SLIDER_KOGGE_STONE : s;
}

int pg_count_moves_batch(const pg_board* pos, uint32_t n, uint32_t* out)
{
    if (!pos || !out) { set_error("null argument"); return PG_ERR_INVALID_ARGUMENT; }
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    if (n == 0) return PG_OK;
    for (u32 i = 0; i < n; i++)
        if (!valid_board(pos[i])) { set_error("position %u is not a valid board", i); return PG_ERR_INVALID_POSITION; }
    return op_batch(0, pos, n, out, nullptr, slider_of(PG_SLIDER_AUTO));
}

int pg_count_moves(const pg_board* pos, uint32_t* out) { return pg_count_moves_batch(pos, 1, out); }

int pg_generate_moves(const pg_board* pos, pg_move* moves, uint32_t* n)
{
    if (!pos || !moves || !n) { set_error("null argument"); return PG_ERR_INVALID_ARGUMENT; }
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    if (!valid_board(*pos)) { set_error("not a valid board"); return PG_ERR_INVALID_POSITION; }
    PG_TRY(op_batch(1, pos, 1, moves, n, slider_of(PG_SLIDER_AUTO)));
    if (*n > 256) { set_error("more than 256 moves"); return PG_ERR_CAPACITY; }
    return PG_OK;
}

int pg_generate_boards(const pg_board* pos, pg_board* out, uint32_t* n)
{
    if (!pos || !out || !n) { set_error("null argument"); return PG_ERR_INVALID_ARGUMENT; }
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    if (!valid_board(*pos)) { set_error("not a valid board"); return PG_ERR_INVALID_POSITION; }
    PG_TRY(op_batch(2, pos, 1, out, n, slider_of(PG_SLIDER_AUTO)));
    if (*n > 256) { set_error("more than 256 boards"); return PG_ERR_CAPACITY; }
    return PG_OK;
}

int pg_make_move(pg_board* pos, pg_move move)
{
    if (!pos) { set_error("null argument"); return PG_ERR_INVALID_ARGUMENT; }
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    PG_TRY(ensure_stage(64));
    Pos* d = (Pos*)E.stage;
    u16* dm = (u16*)((unsigned char*)E.stage + 48);
    PG_CUDA(cudaMemcpyAsync(d, pos, sizeof(Pos), cudaMemcpyHostToDevice, E.stream));
    PG_CUDA(cudaMemcpyAsync(dm, &move, sizeof(u16), cudaMemcpyHostToDevice, E.stream));
    PG_CUDA(g_ops_ks.make_batch(d, dm, 1, E.stream));
    PG_CUDA(cudaMemcpyAsync(pos, d, sizeof(Pos), cudaMemcpyDeviceToHost, E.stream));
    PG_CUDA(cudaStreamSynchronize(E.stream));
    return PG_OK;
}

int pg_random_playouts(uint64_t seed, uint32_t n, int min_plies, int max_plies, int min_moves, int depth_lo,
                       int depth_hi, pg_board* out, uint8_t* depths)
{
    if (!out || n == 0 || min_plies < 0 || max_plies < min_plies || depth_hi < depth_lo || depth_lo < 0 || depth_hi > 15) {
        set_error("bad playout arguments");
        return PG_ERR_INVALID_ARGUMENT;
    }
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    pg_board start;
    pg_board_from_fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1", &start);
    PG_TRY(ensure_stage((u64)n * 49 + 64));
    Pos* d = (Pos*)E.stage;
    unsigned char* dd = (unsigned char*)E.stage + (u64)n * 48;
    PG_CUDA(cudaMemsetAsync(E.err, 0, 4, E.stream));
    Pos sp;
    memcpy(&sp, &start, sizeof(sp));
    PG_CUDA(g_ops_ks.playouts(sp, seed, n, min_plies, max_plies, std::max(min_moves, 1), depth_lo, depth_hi, d,
                              depths ? dd : nullptr, E.err, E.stream));
    PG_CUDA(cudaMemcpyAsync(out, d, (u64)n * 48, cudaMemcpyDeviceToHost, E.stream));
    if (depths) PG_CUDA(cudaMemcpyAsync(depths, dd, n, cudaMemcpyDeviceToHost, E.stream));
    return end_call(nullptr);
}

int pg_autotune(pg_tuning* out)
{
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    if (!E.tuned) {
        E.ticket_next = 0;
        PG_CUDA(cudaMemsetAsync(E.tickets, 0, MAX_TICKETS * sizeof(u32), E.stream));
        PG_TRY(autotune_locked());
    }
    if (out) {
        out->leaf_plies = E.tuned_leaf_plies;
        for (int d = 0; d < 16; d++) {
            out->slider[d] = E.tuned_slider[d];
            out->block_size[d] = E.tuned_T[d];
            out->leaves_per_s[d] = E.tuned_rate[d];
        }
        out->seconds = E.tune_seconds;
    }
    return PG_OK;
}

int pg_perft_split(const pg_board* pos, int depth, int split_plies, pg_move* moves, uint64_t* counts, uint32_t* n,
                   const pg_opts* opts)
{
    if (!pos || !moves || !counts || !n || depth < 1 || depth > 15 || split_plies < 1) {
        set_error("bad argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    PG_TRY(check_opts(opts));
    if (!valid_board(*pos)) {
        set_error("not a valid board");
        return PG_ERR_INVALID_POSITION;
    }
    PG_TRY(begin_call(opts));
    Pos root;
    memcpy(&root, pos, sizeof(root));
    PG_TRY(perft_split_locked(root, depth, split_plies, moves, (u64*)counts, n, opts));
    PG_TRY(end_call(nullptr));
    if (opts && opts->stats) *opts->stats = E.st;
    return PG_OK;
}

int pg_selftest(int which)
{
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    if (which == PG_SELFTEST_BOUNDED_WAIT) return selftest_bounded_wait();
    if (which == PG_SELFTEST_FAIL_NEXT_ALLOC) {
        E.fail_next_alloc = true;
        // drop the level buffers so that the next call must allocate
        cudaStreamSynchronize(E.stream);
        E.alloc_gen++;
        for (auto& lb : E.lv) {
            if (lb.block) cudaFree(lb.block);
            lb = LevelBuf{};
        }
        E.level_bytes_total = 0;
        return PG_OK;
    }
    set_error("unknown self test %d", which);
    return PG_ERR_INVALID_ARGUMENT;
}

int pg_tt_clear(void)
{
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    return tt_clear();
}

int pg_tt_save(const char* path)
{
    if (!path) {
        set_error("null argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    return tt_save(path);
}

int pg_tt_load(const char* path)
{
    if (!path) {
        set_error("null argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    return tt_load(path);
}

int pg_perft_batch_device(const pg_board* d_pos, const uint8_t* d_depths, uint32_t n, uint64_t* d_out,
                          const pg_opts* opts)
{
    if (!d_pos || !d_depths || !d_out) { set_error("null argument"); return PG_ERR_INVALID_ARGUMENT; }
    Engine& E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    PG_TRY(check_opts(opts));
    if (n == 0) return PG_OK;
    PG_TRY(begin_call(opts));
    if (opts && opts->use_tt) {
        PG_TRY(tt_perft_batch_device((const Pos*)d_pos, d_depths, n, (u64*)d_out, opts));
    } else if (opts && opts->graph && opts->persistent) {
        PG_TRY(perft_batch_graph_persistent((const Pos*)d_pos, d_depths, n, (u64*)d_out));
    } else if (opts && opts->graph) {
        PG_TRY(perft_batch_graph_locked((const Pos*)d_pos, d_depths, n, (u64*)d_out, opts));
    } else {
        PG_TRY(perft_batch_device_locked((const Pos*)d_pos, d_depths, n, (u64*)d_out, opts));
    }
    return end_call(opts);
}

int pg_perft_batch(const pg_board* pos, const uint8_t* depths, uint32_t n, uint64_t* out, const pg_opts* opts)
{
    if (!pos || !depths || !out) { set_error("null argument"); return PG_ERR_INVALID_ARGUMENT; }
    Engine& E = engine();
    std::unique_lock<std::mutex> lk(E.mu);
    PG_TRY(check_ready());
    PG_TRY(check_opts(opts));
    if (n == 0) return PG_OK;
    for (u32 i = 0; i < n; i++) {
        if (!valid_board(pos[i])) { set_error("position %u is not a valid board", i); return PG_ERR_INVALID_POSITION; }
        if (depths[i] > 15) { set_error("depth %u of position %u out of range 0..15", depths[i], i); return PG_ERR_INVALID_ARGUMENT; }
    }
    const u64 pb = (u64)n * 48, db = ((u64)n + 15) & ~15ull, ob = (u64)n * 8;
    PG_TRY(ensure_stage(pb + db + ob + 64));
    unsigned char* s = (unsigned char*)E.stage;
    Pos* d_pos = (Pos*)s;
    unsigned char* d_dep = s + pb;
    u64* d_out = (u64*)(s + pb + db);
    PG_TRY(begin_call(opts));
    PG_CUDA(cudaMemcpyAsync(d_pos, pos, pb, cudaMemcpyHostToDevice, E.stream));
    PG_CUDA(cudaMemcpyAsync(d_dep, depths, n, cudaMemcpyHostToDevice, E.stream));
    if (opts && opts->use_tt) {
        PG_TRY(tt_perft_batch_device(d_pos, d_dep, n, d_out, opts));
    } else if (opts && opts->graph && opts->persistent) {
        PG_TRY(perft_batch_graph_persistent(d_pos, d_dep, n, d_out));
    } else if (opts && opts->graph) {
        PG_TRY(perft_batch_graph_locked(d_pos, d_dep, n, d_out, opts));
    } else {
        int maxd = 0;
        for (u32 i = 0; i < n; i++) maxd = std::max<int>(maxd, depths[i]);
        PG_TRY(perft_batch_device_locked(d_pos, d_dep, n, d_out, opts, maxd));
    }
    PG_CUDA(cudaMemcpyAsync(out, d_out, ob, cudaMemcpyDeviceToHost, E.stream));
    PG_TRY(end_call(nullptr));
    u64 total = 0;
    for (u32 i = 0; i < n; i++) total += out[i];
    E.st.leaves = total;
    if (opts && opts->stats) *opts->stats = E.st;
    return PG_OK;
}

int pg_perft(const pg_board* pos, int depth, uint64_t* out, const pg_opts* opts)
{
    if (!pos || !out || depth < 0 || depth > 15) { set_error("bad argument"); return PG_ERR_INVALID_ARGUMENT; }
    const uint8_t d = (uint8_t)depth;
    return pg_perft_batch(pos, &d, 1, out, opts);
}

int pg_perft_divide(const pg_board* pos, int depth, pg_move* moves, uint64_t* counts, uint32_t* n,
                    const pg_opts* opts)
{
    if (!pos || !moves || !counts || !n || depth < 1 || depth > 15) {
        set_error("bad argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    PG_TRY(pg_generate_moves(pos, moves, n));
    if (*n == 0) return PG_OK;
    pg_board kids[256];
    {
        Engine& E = engine();
        std::lock_guard<std::mutex> lk(E.mu);
        PG_TRY(ensure_stage(256 * 48 + 512 + 64));
        Pos* d = (Pos*)E.stage;
        u16* dm = (u16*)((unsigned char*)E.stage + 256 * 48);
        for (u32 i = 0; i < *n; i++) kids[i] = *pos;
        PG_CUDA(cudaMemcpyAsync(d, kids, *n * 48, cudaMemcpyHostToDevice, E.stream));
        PG_CUDA(cudaMemcpyAsync(dm, moves, *n * 2, cudaMemcpyHostToDevice, E.stream));
        PG_CUDA(g_ops_ks.make_batch(d, dm, *n, E.stream));
        PG_CUDA(cudaMemcpyAsync(kids, d, *n * 48, cudaMemcpyDeviceToHost, E.stream));
        PG_CUDA(cudaStreamSynchronize(E.stream));
    }
    uint8_t dep[256];
    for (u32 i = 0; i < *n; i++) dep[i] = (uint8_t)(depth - 1);
    return pg_perft_batch(kids, dep, *n, counts, opts);
}

}  // extern "C"
