// pg_engine.cuh -- engine state shared by the translation units of the
// library (host side) and the kernel interfaces they launch.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/perft_gb300.h"
#include "pg_board.cuh"

namespace pg {

constexpr int MAX_LEVELS = 16;
// device bytes per node of a level buffer: the board (48), group id (4),
// remaining depth (1), child count (4) and scanned offset (8)
constexpr u64 LEVEL_NODE_BYTES = 48 + 4 + 1 + 4 + 8;
constexpr u32 MAX_CHUNKS = 2048;      // greedy chunks planned per expansion
constexpr u32 MAX_TICKETS = 1 << 16;  // dynamic-scheduling counters per call

// device error bits (bounded waits and capacity guards set them; no trap)
enum : u32 {
    ERR_SCAN_TIMEOUT = 1u << 0,
    ERR_PLAN_OVERFLOW = 1u << 1,
    ERR_PLAYOUT_ATTEMPTS = 1u << 2,
    ERR_QUEUE_MISMATCH = 1u << 3,
    ERR_GRID_BARRIER_TIMEOUT = 1u << 4,
    ERR_TT_GUARD = 1u << 5,
    ERR_LEVEL_CAP = 1u << 6,  // a persistent launch reached a level the host did not prepare
};

// one frontier level in HBM: boards as three 16-byte planes (struct of
// arrays, one ulonglong2 per board per plane), group id and remaining depth
struct LevelView {
    ulonglong2* pl0;  // (white, pawns)
    ulonglong2* pl1;  // (knights, bishop_queens)
    ulonglong2* pl2;  // (rook_queens, kings)
    u32* grp;
    unsigned char* rem;
};

struct LevelBuf {
    LevelView v{};
    u32* cnt = nullptr;   // children per node (0 for leaf-handled nodes)
    u64* offs = nullptr;  // exclusive scan of cnt, cap + 1 entries
    u64 cap = 0;
    void* block = nullptr;
};

struct PlanOut {
    u32 nchunks;
    u32 pad;
    u64 total;
    u32 bnd[MAX_CHUNKS + 1];
    u64 coff[MAX_CHUNKS + 1];  // offs[] at each boundary
};

enum PlanMode { PLAN_NONE = 0, PLAN_RECORD = 1, PLAN_REPLAY = 2 };

// control words of one persistent launch (pg_persist.cuh; device memory,
// zeroed by the host before the launch, part[2] = 0xFFFFFFFF): grid barrier
// arrival count and generation, abort flag, root partition counters (white,
// black, min depth, max depth)
struct PersistCtl {
    u32 bar_count, bar_gen, abort, pad;
    u32 part[4];
};

// arguments of one persistent launch: the roots, the level buffers the host
// prepared (cap 0 = not prepared), per-level chunk plans, scan status words,
// phase tickets (zeroed), control words, error bits
struct PersistArgs {
    const Pos* pos;
    const unsigned char* depths;
    const u32* groups;  // group id per root (null: the root's index)
    u32 n;
    u64* acc;  // per-group counts (added to)
    LevelView lv[MAX_LEVELS];
    u32* cnt[MAX_LEVELS];
    u64* offs[MAX_LEVELS];
    u64 cap[MAX_LEVELS];
    PlanOut* plan;  // MAX_LEVELS plans
    u64* status;
    u64 status_cap;
    u32* tickets;
    u32 max_tickets;
    PersistCtl* ctl;
    u32* err;
};
// the persistent launch (Kogge-Stone translation unit); *grid = CTAs launched
cudaError_t persist_launch(const PersistArgs& a, cudaStream_t st, int num_sms, int* grid);
constexpr int PERSIST_CTA = 128;  // threads per CTA of the persistent launch
constexpr u32 PERSIST_SCAN_TILE_NODES = 1024;  // counts per scan tile of the persistent launch

// one captured batch (see perft_batch_graph_locked)
struct GraphCache {
    cudaGraphExec_t exec = nullptr;
    const void* pos = nullptr;
    const void* dep = nullptr;
    const void* out = nullptr;
    u32 n = 0;
    u64 sum = 0;
    int slider = 0, T = 0, leaf_plies = 0;
    bool per_depth = false;
    u64 launches = 0;
    u64 alloc_gen = 0;  // Engine::alloc_gen when captured
    bool persistent = false;  // one persistent launch: valid for any contents of the same size and largest depth
    int maxd = 0;
};

struct Engine {
    std::mutex mu;
    bool ready = false;
    int device = 0;
    int num_sms = 0;
    int verbose = 0;
    int default_slider = PG_SLIDER_AUTO;
    u64 budget = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // start/end event pairs around leaf launches, read after the next host
    // synchronisation instead of waiting on each launch
    std::vector<cudaEvent_t> leaf_ev;
    size_t leaf_ev_used = 0;
    LevelBuf lv[MAX_LEVELS];
    u64 level_bytes_total = 0;
    // scratch
    u64* scan_status = nullptr;
    u64 scan_status_cap = 0;
    u32* tickets = nullptr;  // MAX_TICKETS counters, zeroed per call
    u32 ticket_next = 0;
    u32* err = nullptr;
    PlanOut* plan_dev = nullptr;
    PlanOut* plan_host = nullptr;  // pinned
    u64* acc = nullptr;            // per-group counters
    u64 acc_cap = 0;
    void* stage = nullptr;         // staging for host-array calls
    u64 stage_cap = 0;
    u64* host_scratch = nullptr;   // pinned small scratch
    u64* aux = nullptr;            // small device scratch (input checksum)
    PlanOut* persist_plan = nullptr;  // MAX_LEVELS chunk plans of a persistent launch
    PersistCtl* persist_ctl = nullptr;
    // launch-plan recording for graph capture
    int plan_mode = PLAN_NONE;
    std::vector<std::vector<u32>> rec_bnd;
    std::vector<std::vector<u64>> rec_off;
    size_t rec_next = 0;
    u32 rec_part[4] = {};
    GraphCache graph;
    // bumped whenever a device buffer that a captured graph may name (level
    // buffers, scan status words, the staging buffer) is freed or
    // reallocated; a cached graph from an older generation is re-captured
    u64 alloc_gen = 0;
    // statistics of the current call
    pg_stats st{};
    // autotuner result: best leaf variant per root depth, switch depth
    bool tuned = false;
    int tuned_leaf_plies = 2;
    int tuned_slider[16] = {};
    int tuned_T[16] = {};
    double tuned_rate[16] = {};
    double tune_seconds = 0;
    // host-side fault injection for tests: the next level allocation fails
    bool fail_next_alloc = false;
};

Engine& engine();
void set_error(const char* fmt, ...);

// engine internals shared by the translation units (call with engine().mu held)
struct Variant {
    int slider = PG_SLIDER_KOGGE_STONE;  // pg_slider (never AUTO here)
    int T = 256;                         // CTA size of the block-queue kernels
    int leaf_plies = 2;                  // plies finished inside one CTA (switch depth)
    bool per_depth = false;              // take the leaf kernel's slider/T from the tuning table
};
Variant pick_variant(const pg_opts* o);
u32* next_ticket();
int launch_leaf(const Variant& v, int side, const LevelView& lv, u32 start, u32 n, u64* acc);
int launch_expand(const Variant& v, int side, const LevelView& in, u32 start, u32 a, u32 b, const u64* offs,
                  const LevelView& out);
int launch_count(const Variant& v, int side, const LevelView& lv, u32 start, u32 n, u32* cnt);
int launch_scan(const u32* cnt, u32 n, u64* offs);
u64 level_cap_max();
int ensure_level(int L, u64 need);
int ensure_stage(u64 bytes);
int perft_core(const Pos* d_pos, const unsigned char* d_depths, const u32* d_groups, u32 n, u64* acc, bool zero_acc,
               const Variant& v);
int expand_frontier(const Pos& root, int plies, Pos* out, u32 cap, u32* n_out);
int perft_core_persistent(const Pos* d_pos, const unsigned char* d_depths, const u32* d_groups, u32 n, u64* acc,
                          bool zero_acc, int maxd);

}  // namespace pg
