// pg_tt.cu -- perft with Zobrist transposition tables in HBM.
//
// The reference's TT path (perft_bb_gpu_simple_hash, perft_bb.h:1242-1589;
// entries chess.h:410-504; probes perft_bb.h:664-761; duplicate marking
// perft_bb.h:790-852; upsweep and stores perft_bb.h:854-961) re-planned for
// the chunked breadth-first driver:
//   * keys: 128-bit Zobrist keys (pg_zobrist.cuh: two seeded 64-bit words
//     per feature, the shape of the reference's HashKey128b), computed in
//     full at the root level and below it updated from the parent's key by
//     the features the move changed (the reference updates them in makeMove);
//   * one table per remaining depth 2..9 of 32-byte entries that carry the
//     count XORed into all 128 key bits (pg_zobrist.cuh), written as two
//     16-byte stores; a foreign or torn entry is a miss, never a wrong count
//     (the reference's lockless XOR scheme, widened to the whole key);
//   * per level: probe (a hit resolves the node), duplicate detection inside
//     the level (first claim in a level table by a 64-bit digest; a later
//     node takes the claimant's count only if its full 128-bit key and
//     remaining depth are equal), the usual leaf / count / scan / expand for
//     the live nodes, and after each chunk an upsweep that stores the
//     children's final counts and adds them into their parents;
//   * use_tt = 2 (PG_TT_DEDUP_ONLY) runs the same driver without the HBM
//     tables: only the in-level duplicate pass.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "pg_kernels.cuh"
#include "pg_tables.h"
#include "pg_tt.cuh"
#include "pg_zobrist.cuh"

namespace pg {

constexpr int TT_MIN_DEPTH = 2, TT_MAX_DEPTH = 9;
constexpr u32 NO_DUP = 0xFFFFFFFFu;
constexpr u64 TT_ENTRY_BYTES = 32;

static __device__ ulonglong2 g_zobrist[ZOBRIST_KEYS];

// tab[d]: the table of remaining depth d, two ulonglong2 per entry (entry i
// at tab[d][2i], tab[d][2i + 1]); null when that depth has no table
struct TTSet {
    ulonglong2* tab[16];
    u64 mask[16];
};

struct LevelTT {
    u64* hash0 = nullptr;  // 128-bit key of each node, low / high word
    u64* hash1 = nullptr;
    u64* acc = nullptr;
    u32* parent = nullptr;
    u32* dup = nullptr;
    u64* dd_hash = nullptr;  // duplicate table of the level
    u32* dd_idx = nullptr;
    u64 cap = 0, dd_cap = 0;
    void* block = nullptr;
};

struct TTState {
    bool keys_ready = false;
    TTSet set{};     // the HBM tables
    TTSet active{};  // what the current call probes and stores: set, or none (PG_TT_DEDUP_ONLY)
    void* pool = nullptr;
    u64 pool_bytes = 0;
    LevelTT lv[MAX_LEVELS];
    u32* root_of = nullptr;
    u64 root_cap = 0;
    u64* counters = nullptr;  // probes, hits, stores
};
static TTState g_tt;

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// the duplicate table's 64-bit digest of (key, remaining depth): one level of
// a mixed-depth batch can hold the same position at different depths.  The
// digest only finds the slot and the claimant; equality is decided on the
// full key and depth (k_tt_dedup).
__device__ __forceinline__ u64 dd_key(u64 h, u32 rem)
{
    const u64 k = h ^ (0x9E3779B97F4A7C15ull * (rem + 1));
    return k ? k : 1;
}
// slot of a digest in a table of `slots` entries (any size): the high word of
// digest x slots, after a multiply that spreads every digest bit upward
__device__ __forceinline__ u32 dd_slot(u64 k, u64 slots)
{
    return (u32)__umul64hi(k * 0xD6E8FEB86659FD93ull ^ (k >> 32), slots);
}

// Adds a per-thread count into *dst with one global atomic per CTA (the
// threads of a warp are summed by a warp reduction, the warps in shared
// memory); every thread of the CTA calls it.
__device__ __forceinline__ void block_count_add(u64* dst, u32 v)
{
    __shared__ u32 s_sum;
    if (threadIdx.x == 0) s_sum = 0;
    __syncthreads();
    const u32 w = __reduce_add_sync(0xFFFFFFFFu, v);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&s_sum, w);
    __syncthreads();
    if (threadIdx.x == 0 && s_sum) atomicAdd(dst, (u64)s_sum);
}

// the parent level of a level below the root, as the probe reads it: its
// boards and keys, and each node's parent slot (parent null at the root level)
struct ParentKeys {
    LevelView lv;
    const u64* hash0;
    const u64* hash1;
    const u32* parent;
};

// key, TT probe, and first claim of the level's duplicate table.  Below the
// root level a node's key is its parent's key updated by the features the
// move changed (the parent was probed one level up: a child that reaches
// the probe has remaining depth >= TT_MIN_DEPTH, so its parent had more
// and its key was written); at the root level the key is computed in full.
static __global__ void k_tt_probe(LevelView lv, u32 start, u32 n, LevelTT lt, ParentKeys pk, TTSet tt, u64 dd_slots,
                                  u64* counters)
{
    __shared__ ulonglong2 z[ZOBRIST_KEYS];
    for (int i = threadIdx.x; i < ZOBRIST_KEYS; i += blockDim.x) z[i] = g_zobrist[i];
    __syncthreads();
    u32 probes = 0, hits = 0;
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const u32 idx = start + i;
        const u32 rem = lv.rem[idx];
        lt.acc[idx] = 0;
        lt.dup[idx] = NO_DUP;
        if (rem < TT_MIN_DEPTH || rem >= REM_DEAD) continue;
        const Pos b = load_board(lv, idx);
        ulonglong2 h;
        if (pk.parent) {
            const u32 p = pk.parent[idx];
            const Pos pb = load_board(pk.lv, p);
            h = zobrist128_from(&pb.w, make_ulonglong2(pk.hash0[p], pk.hash1[p]), &b.w, z);
        } else {
            h = zobrist128(&b.w, z);
        }
        lt.hash0[idx] = h.x;
        lt.hash1[idx] = h.y;
        if (rem <= TT_MAX_DEPTH && tt.tab[rem]) {
            probes++;
            const ulonglong2* e = tt.tab[rem] + 2 * (h.x & tt.mask[rem]);
            const ulonglong2 ea = e[0], eb = e[1];
            u64 v;
            if (tt_match(ea, eb, h.x, h.y, v)) {
                lt.acc[idx] = v;
                lv.rem[idx] = REM_DEAD;
                hits++;
                continue;
            }
        }
        const u64 k = dd_key(h.x, rem);
        const u32 s = dd_slot(k, dd_slots);
        const u64 prev = atomicCAS(&lt.dd_hash[s], 0ull, k);
        if (prev == 0 || prev == k) atomicMin(&lt.dd_idx[s], idx);
    }
    block_count_add(&counters[0], probes);
    block_count_add(&counters[1], hits);
}

// a node whose position and remaining depth were claimed first by another
// node of its level takes that node's count later and does no work itself.
// The claimant of a slot is the lowest index among the nodes with the
// slot's digest; a node whose full key or depth differs from the claimant's
// (a digest collision) keeps its own work.  Claimants are never marked here,
// so their depth and key are stable while others compare against them.
static __global__ void k_tt_dedup(LevelView lv, u32 start, u32 n, LevelTT lt, u64 dd_slots)
{
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const u32 idx = start + i;
        const u32 rem = lv.rem[idx];
        if (rem < TT_MIN_DEPTH || rem >= REM_DEAD) continue;
        const u64 h0 = lt.hash0[idx];
        const u64 k = dd_key(h0, rem);
        const u32 s = dd_slot(k, dd_slots);
        if (lt.dd_hash[s] == k) {
            const u32 rep = lt.dd_idx[s];
            if (rep != idx && lt.hash0[rep] == h0 && lt.hash1[rep] == lt.hash1[idx] && lv.rem[rep] == rem) {
                lt.dup[idx] = rep;
                lv.rem[idx] = REM_DEAD;
            }
        }
    }
}

__device__ __forceinline__ void tt_store(const TTSet& tt, u32 rem, u64 h0, u64 h1, u64 v)
{
    ulonglong2 a, b;
    tt_pack(h0, h1, v, a, b);
    ulonglong2* e = tt.tab[rem] + 2 * (h0 & tt.mask[rem]);
    e[0] = a;
    e[1] = b;
}

// children [0, m) of one chunk are final: store them and add them to parents.
// The expansion writes the children of a parent next to each other in parent
// order, so a warp sums each run of equal parents (segmented shuffle
// reduction) and adds it with one atomic; a warp whose parents are not in
// order adds lane by lane.
static __global__ void k_tt_upsweep(LevelView ch, u32 m, LevelTT ct, TTSet tt, u64* __restrict__ parent_acc,
                                    u64* counters)
{
    constexpr unsigned FULL = 0xFFFFFFFFu;
    const u32 lane = threadIdx.x & 31;
    const u32 stride = gridDim.x * blockDim.x;  // a multiple of 32: every lane of a warp runs the same iterations
    u32 stores = 0;
    for (u32 base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < m; base += stride) {
        const u32 j = base + lane;
        const bool valid = j < m;
        u64 v = 0;
        u32 par = 0xFFFFFFFFu;
        if (valid) {
            const u32 d = ct.dup[j];
            v = d != NO_DUP ? ct.acc[d] : ct.acc[j];
            const u32 rem = ch.rem[j];
            if (rem >= TT_MIN_DEPTH && rem <= TT_MAX_DEPTH && tt.tab[rem]) {
                tt_store(tt, rem, ct.hash0[j], ct.hash1[j], v);
                stores++;
            }
            par = ct.parent[j];
        }
        const u32 prev = __shfl_up_sync(FULL, par, 1);
        const u32 next = __shfl_down_sync(FULL, par, 1);
        if (!__all_sync(FULL, lane == 31 || next >= par)) {
            if (valid) atomicAdd(&parent_acc[par], v);
            continue;
        }
        for (u32 o = 1; o < 32; o <<= 1) {
            const u64 vn = __shfl_down_sync(FULL, v, o);
            const u32 pn = __shfl_down_sync(FULL, par, o);
            if (lane + o < 32 && pn == par) v += vn;
        }
        if (valid && (lane == 0 || prev != par)) atomicAdd(&parent_acc[par], v);
    }
    block_count_add(&counters[2], stores);
}

// level 0: remember each slot's root, make each slot its own group
static __global__ void k_tt_roots(LevelView lv, u32 n, u32* __restrict__ root_of)
{
    for (u32 s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        root_of[s] = lv.grp[s];
        lv.grp[s] = s;
    }
}

static __global__ void k_tt_finish(LevelView lv, u32 n, LevelTT lt, TTSet tt, const u32* __restrict__ root_of,
                                   u64* __restrict__ out, u64* counters)
{
    u32 stores = 0;
    for (u32 s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const u32 d = lt.dup[s];
        const u64 v = d != NO_DUP ? lt.acc[d] : lt.acc[s];
        const u32 rem = lv.rem[s];
        if (rem >= TT_MIN_DEPTH && rem <= TT_MAX_DEPTH && tt.tab[rem]) {
            tt_store(tt, rem, lt.hash0[s], lt.hash1[s], v);
            stores++;
        }
        out[root_of[s]] = v;
    }
    block_count_add(&counters[2], stores);
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------

#define TT_CUDA(call)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? PG_ERR_OUT_OF_MEMORY : PG_ERR_CUDA;    \
        }                                                                                    \
    } while (0)
#define TT_TRY(expr)                  \
    do {                              \
        int r_ = (expr);              \
        if (r_ != PG_OK) return r_;   \
    } while (0)

static int small_grid(u64 n) { return (int)std::max<u64>(1, std::min<u64>((n + 255) / 256, 8192)); }

int tt_upload_keys()
{
    ulonglong2 keys[ZOBRIST_KEYS];
    zobrist_key_table(keys);
    TT_CUDA(cudaMemcpyToSymbol(g_zobrist, keys, sizeof(keys)));
    const HostTables* t = host_tables();
    if (!t) {
        set_error("table construction failed");
        return PG_ERR_CUDA;
    }
    TT_CUDA(upload_static_tables(*t));
    g_tt.keys_ready = true;
    return PG_OK;
}

static int ensure_tables(u64 bytes)
{
    Engine& E = engine();
    if (g_tt.pool && g_tt.pool_bytes == bytes) return PG_OK;
    if (g_tt.pool) {
        cudaFree(g_tt.pool);
        g_tt.pool = nullptr;
        g_tt.set = TTSet{};
    }
    const int ntab = TT_MAX_DEPTH - TT_MIN_DEPTH + 1;
    u64 entries = 1;
    while (entries * 2 * TT_ENTRY_BYTES * ntab <= bytes) entries *= 2;
    if (entries < 1024) {
        set_error("transposition-table budget of %llu bytes is too small", (unsigned long long)bytes);
        return PG_ERR_INVALID_ARGUMENT;
    }
    TT_CUDA(cudaMalloc(&g_tt.pool, entries * TT_ENTRY_BYTES * ntab));
    TT_CUDA(cudaMemsetAsync(g_tt.pool, 0, entries * TT_ENTRY_BYTES * ntab, E.stream));
    g_tt.pool_bytes = bytes;
    for (int d = TT_MIN_DEPTH; d <= TT_MAX_DEPTH; d++) {
        g_tt.set.tab[d] = (ulonglong2*)g_tt.pool + (u64)(d - TT_MIN_DEPTH) * entries * 2;
        g_tt.set.mask[d] = entries - 1;
    }
    if (!g_tt.counters) TT_CUDA(cudaMalloc(&g_tt.counters, 4 * sizeof(u64)));
    return PG_OK;
}

// per node of a level in the TT driver, beside the level buffer: both key
// words, the count, the parent slot and the duplicate index (32 B), and two
// slots of the level's duplicate table (12 B each)
constexpr u64 TT_NODE_BYTES = 32 + 2 * 12;

// nodes a level of the TT driver holds: a quarter of the HBM budget left
// beside the tables, over the level buffer's and the TT metadata's bytes
// per node (the same share as level_cap_max gives the driver without TT)
static u64 tt_level_cap()
{
    Engine& E = engine();
    const u64 avail = E.budget > g_tt.pool_bytes ? E.budget - g_tt.pool_bytes : E.budget / 4;
    const u64 cap = std::min<u64>(avail / (LEVEL_NODE_BYTES + TT_NODE_BYTES) / 4, level_cap_max());
    return std::max<u64>(cap, 1u << 16);
}

// sized to the nodes asked for (a multiple of 65,536), not the next power
// of two: at the largest levels the rounding alone would double the bytes
static int ensure_level_tt(int L, u64 need)
{
    LevelTT& t = g_tt.lv[L];
    if (t.cap >= need) return PG_OK;
    if (t.block) {
        TT_CUDA(cudaStreamSynchronize(engine().stream));
        cudaFree(t.block);
        t = LevelTT{};
    }
    const u64 cap = std::max<u64>(1u << 16, (need + 65535) & ~65535ull);
    const u64 dd = 2 * cap;
    const u64 bytes = cap * (8 + 8 + 8 + 4 + 4) + dd * (8 + 4) + 1024;
    void* blk = nullptr;
    cudaError_t e = cudaMalloc(&blk, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("transposition-table level %d of %llu nodes failed: %s", L, (unsigned long long)cap,
                  cudaGetErrorString(e));
        return PG_ERR_OUT_OF_MEMORY;
    }
    unsigned char* p = (unsigned char*)blk;
    t.hash0 = (u64*)p;
    p += cap * 8;
    t.hash1 = (u64*)p;
    p += cap * 8;
    t.acc = (u64*)p;
    p += cap * 8;
    t.dd_hash = (u64*)p;
    p += dd * 8;
    t.parent = (u32*)p;
    p += cap * 4;
    t.dup = (u32*)p;
    p += cap * 4;
    t.dd_idx = (u32*)p;
    t.cap = cap;
    t.dd_cap = dd;
    t.block = blk;
    return PG_OK;
}

static int run_range_tt(const Variant& v, int L, u32 start, u32 n, int side, int minrem, int maxrem)
{
    Engine& E = engine();
    if (n == 0) return PG_OK;
    LevelBuf& lb = E.lv[L];
    LevelTT& lt = g_tt.lv[L];
    // two duplicate-table slots per node of the range (the table is sized for
    // the level's capacity)
    const u64 dd = std::min(std::max<u64>(1024, 2ull * n), lt.dd_cap);
    TT_CUDA(cudaMemsetAsync(lt.dd_hash, 0, dd * 8, E.stream));
    TT_CUDA(cudaMemsetAsync(lt.dd_idx, 0xFF, dd * 4, E.stream));
    ParentKeys pk{};
    if (L > 0) pk = {E.lv[L - 1].v, g_tt.lv[L - 1].hash0, g_tt.lv[L - 1].hash1, lt.parent};
    k_tt_probe<<<small_grid(n), 256, 0, E.stream>>>(lb.v, start, n, lt, pk, g_tt.active, dd, g_tt.counters);
    k_tt_dedup<<<small_grid(n), 256, 0, E.stream>>>(lb.v, start, n, lt, dd);
    TT_CUDA(cudaGetLastError());
    E.st.launches += 2;
    if (minrem <= 2) TT_TRY(launch_leaf(v, side, lb.v, start, n, lt.acc));
    if (maxrem < 3) return PG_OK;
    TT_TRY(launch_count(v, side, lb.v, start, n, lb.cnt));
    TT_TRY(launch_scan(lb.cnt, n, lb.offs));
    const u64 cap_next = tt_level_cap();
    k_plan<<<1, 32, 0, E.stream>>>(lb.offs, n, cap_next, E.plan_dev, E.err);
    TT_CUDA(cudaGetLastError());
    TT_CUDA(cudaMemcpyAsync(E.plan_host, E.plan_dev, sizeof(PlanOut), cudaMemcpyDeviceToHost, E.stream));
    TT_CUDA(cudaStreamSynchronize(E.stream));
    const PlanOut plan = *E.plan_host;
    std::vector<u32> bnd(plan.bnd, plan.bnd + plan.nchunks + 1);
    std::vector<u64> boff(plan.coff, plan.coff + plan.nchunks + 1);
    const int cminrem = std::max(minrem, 3) - 1, cmaxrem = maxrem - 1;
    for (size_t k = 0; k + 1 < bnd.size(); k++) {
        const u64 children = boff[k + 1] - boff[k];
        if (!children) continue;
        TT_TRY(ensure_level(L + 1, children));
        TT_TRY(ensure_level_tt(L + 1, children));
        u32* tk = next_ticket();
        if (!tk) {
            set_error("dynamic-scheduling counters exhausted");
            return PG_ERR_CAPACITY;
        }
        constexpr int T = 256, Q = T * 32;
        using BL = BlockSmem<SlKS, T, Q>;
        const int grid = std::min<u64>((bnd[k + 1] - bnd[k] + T - 1) / T, (u64)E.num_sms * 2);
        if (side)
            k_expand<1, SlKS, T, Q><<<std::max(grid, 1), T, BL::bytes, E.stream>>>(
                lb.v, start, bnd[k], bnd[k + 1], lb.offs, E.lv[L + 1].v, tk, g_tt.lv[L + 1].parent);
        else
            k_expand<0, SlKS, T, Q><<<std::max(grid, 1), T, BL::bytes, E.stream>>>(
                lb.v, start, bnd[k], bnd[k + 1], lb.offs, E.lv[L + 1].v, tk, g_tt.lv[L + 1].parent);
        TT_CUDA(cudaGetLastError());
        E.st.launches++;
        TT_TRY(run_range_tt(v, L + 1, 0, (u32)children, 1 - side, cminrem, cmaxrem));
        k_tt_upsweep<<<small_grid(children), 256, 0, E.stream>>>(E.lv[L + 1].v, (u32)children, g_tt.lv[L + 1],
                                                                 g_tt.active, lt.acc, g_tt.counters);
        TT_CUDA(cudaGetLastError());
        E.st.launches++;
    }
    return PG_OK;
}

void tt_free()
{
    if (g_tt.pool) cudaFree(g_tt.pool);
    for (auto& t : g_tt.lv) {
        if (t.block) cudaFree(t.block);
        t = LevelTT{};
    }
    if (g_tt.root_of) cudaFree(g_tt.root_of);
    if (g_tt.counters) cudaFree(g_tt.counters);
    g_tt = TTState{};
}

// ---------------------------------------------------------------------------
// snapshot of the tables on disk.  The reference keeps a chained table in a
// file and probes it during the search (diskTTProbe, launcher.h:699-790, off
// by default); here the HBM tables are written out whole and read back, so a
// later process starts with the subtrees an earlier one counted.  The file is
// a header (format, Zobrist seeds, depth range, entries per table, the TT
// size the tables were made for) followed by the tables as they lie in HBM.
// ---------------------------------------------------------------------------

struct TTFileHeader {
    char magic[8];       // "PGTT" and the format version
    u64 key_seed[2];     // entries are only valid under the same keys
    u32 min_depth, max_depth;
    u64 entries;         // per table (a power of two)
    u64 budget_bytes;    // the TT size the tables were made for
};
// format 2: 128-bit keys, 32-byte entries
static const char TT_MAGIC[8] = {'P', 'G', 'T', 'T', 0, 0, 0, 2};
constexpr u64 TT_FILE_CHUNK = 64ull << 20;

int tt_save(const char* path)
{
    Engine& E = engine();
    if (!g_tt.pool) {
        set_error("no transposition tables to save (run a perft with use_tt first)");
        return PG_ERR_INVALID_ARGUMENT;
    }
    TT_CUDA(cudaStreamSynchronize(E.stream));
    const int ntab = TT_MAX_DEPTH - TT_MIN_DEPTH + 1;
    TTFileHeader h{};
    memcpy(h.magic, TT_MAGIC, sizeof(h.magic));
    h.key_seed[0] = ZOBRIST_SEED0;
    h.key_seed[1] = ZOBRIST_SEED1;
    h.min_depth = TT_MIN_DEPTH;
    h.max_depth = TT_MAX_DEPTH;
    h.entries = g_tt.set.mask[TT_MIN_DEPTH] + 1;
    h.budget_bytes = g_tt.pool_bytes;
    const u64 total = h.entries * TT_ENTRY_BYTES * ntab;
    FILE* f = fopen(path, "wb");
    if (!f) {
        set_error("cannot open %s for writing", path);
        return PG_ERR_INVALID_ARGUMENT;
    }
    std::vector<unsigned char> buf((size_t)std::min(total, TT_FILE_CHUNK));
    bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
    for (u64 off = 0; ok && off < total; off += TT_FILE_CHUNK) {
        const u64 len = std::min(TT_FILE_CHUNK, total - off);
        // on the engine's stream, completed before the buffer is written out
        cudaError_t e = cudaMemcpyAsync(buf.data(), (unsigned char*)g_tt.pool + off, len, cudaMemcpyDeviceToHost,
                                        E.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(E.stream);
        if (e != cudaSuccess) {
            fclose(f);
            set_error("reading the tables failed: %s", cudaGetErrorString(e));
            return PG_ERR_CUDA;
        }
        ok = fwrite(buf.data(), 1, len, f) == len;
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok) {
        set_error("writing %s failed", path);
        return PG_ERR_INVALID_ARGUMENT;
    }
    return PG_OK;
}

int tt_load(const char* path)
{
    Engine& E = engine();
    FILE* f = fopen(path, "rb");
    if (!f) {
        set_error("cannot open %s", path);
        return PG_ERR_INVALID_ARGUMENT;
    }
    TTFileHeader h{};
    const int ntab = TT_MAX_DEPTH - TT_MIN_DEPTH + 1;
    if (fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, TT_MAGIC, sizeof(h.magic)) != 0 ||
        h.key_seed[0] != ZOBRIST_SEED0 || h.key_seed[1] != ZOBRIST_SEED1 || h.min_depth != (u32)TT_MIN_DEPTH || h.max_depth != (u32)TT_MAX_DEPTH ||
        h.entries < 1024 || (h.entries & (h.entries - 1))) {
        fclose(f);
        set_error("%s is not a transposition-table snapshot of this engine", path);
        return PG_ERR_INVALID_ARGUMENT;
    }
    if (!g_tt.keys_ready) {
        const int r = tt_upload_keys();
        if (r != PG_OK) {
            fclose(f);
            return r;
        }
    }
    {
        const int r = ensure_tables(h.budget_bytes);
        if (r != PG_OK || g_tt.set.mask[TT_MIN_DEPTH] + 1 != h.entries) {
            fclose(f);
            if (r == PG_OK) set_error("%s: table layout does not match", path);
            return r != PG_OK ? r : PG_ERR_INVALID_ARGUMENT;
        }
    }
    const cudaError_t se = cudaStreamSynchronize(E.stream);
    if (se != cudaSuccess) {
        fclose(f);
        set_error("cudaStreamSynchronize failed: %s", cudaGetErrorString(se));
        return PG_ERR_CUDA;
    }
    const u64 total = h.entries * TT_ENTRY_BYTES * ntab;
    std::vector<unsigned char> buf((size_t)std::min(total, TT_FILE_CHUNK));
    for (u64 off = 0; off < total; off += TT_FILE_CHUNK) {
        const u64 len = std::min(TT_FILE_CHUNK, total - off);
        if (fread(buf.data(), 1, len, f) != len) {
            fclose(f);
            // never leave half a snapshot
            if (cudaMemsetAsync(g_tt.pool, 0, total, E.stream) == cudaSuccess) cudaStreamSynchronize(E.stream);
            set_error("%s is shorter than its header says", path);
            return PG_ERR_INVALID_ARGUMENT;
        }
        // on the engine's stream (the engine's kernels run on a non-blocking
        // stream), completed before the buffer is reused
        cudaError_t e = cudaMemcpyAsync((unsigned char*)g_tt.pool + off, buf.data(), len, cudaMemcpyHostToDevice,
                                        E.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(E.stream);
        if (e != cudaSuccess) {
            fclose(f);
            set_error("writing the tables failed: %s", cudaGetErrorString(e));
            return PG_ERR_CUDA;
        }
    }
    fclose(f);
    return PG_OK;
}

int tt_clear()
{
    Engine& E = engine();
    if (g_tt.pool) {
        const u64 bytes = (g_tt.set.mask[TT_MIN_DEPTH] + 1) * TT_ENTRY_BYTES * (TT_MAX_DEPTH - TT_MIN_DEPTH + 1);
        TT_CUDA(cudaMemsetAsync(g_tt.pool, 0, bytes, E.stream));
    }
    TT_CUDA(cudaStreamSynchronize(E.stream));
    return PG_OK;
}

int tt_perft_batch_device(const Pos* d_pos, const unsigned char* d_depths, u32 n, u64* d_out, const pg_opts* o)
{
    Engine& E = engine();
    if (!g_tt.keys_ready) TT_TRY(tt_upload_keys());
    const bool tables = !(o && o->use_tt == PG_TT_DEDUP_ONLY);
    if (tables) {
        const u64 bytes = (o && o->tt_bytes) ? o->tt_bytes : std::min<u64>(32ull << 30, E.budget / 4);
        TT_TRY(ensure_tables(bytes));
        g_tt.active = g_tt.set;
    } else {
        g_tt.active = TTSet{};
    }
    if (!g_tt.counters) TT_CUDA(cudaMalloc(&g_tt.counters, 4 * sizeof(u64)));
    Variant v = pick_variant(o);
    v.leaf_plies = 2;  // the TT driver finishes the last two plies in the leaf kernel
    TT_TRY(ensure_level(0, n));
    TT_TRY(ensure_level_tt(0, n));
    if (g_tt.root_cap < n) {
        if (g_tt.root_of) cudaFree(g_tt.root_of);
        g_tt.root_of = nullptr;
        TT_CUDA(cudaMalloc(&g_tt.root_of, (u64)n * 4));
        g_tt.root_cap = n;
    }
    TT_CUDA(cudaMemsetAsync(g_tt.counters, 0, 4 * sizeof(u64), E.stream));
    u32* ctr = (u32*)(E.host_scratch + 64);
    u32* dctr = E.tickets + MAX_TICKETS - 4;
    const u32 init[4] = {0, 0, 0xFFFFFFFFu, 0};
    TT_CUDA(cudaMemcpyAsync(dctr, init, sizeof(init), cudaMemcpyHostToDevice, E.stream));
    k_partition_roots<<<small_grid(n), 256, 0, E.stream>>>(d_pos, d_depths, n, E.lv[0].v, dctr, nullptr);
    k_tt_roots<<<small_grid(n), 256, 0, E.stream>>>(E.lv[0].v, n, g_tt.root_of);
    TT_CUDA(cudaGetLastError());
    TT_CUDA(cudaMemcpyAsync(ctr, dctr, 4 * sizeof(u32), cudaMemcpyDeviceToHost, E.stream));
    TT_CUDA(cudaStreamSynchronize(E.stream));
    const u32 nw = ctr[0], mind = ctr[2], maxd = ctr[3];
    if (maxd > 15) {
        set_error("depth %u out of range 0..15", maxd);
        return PG_ERR_INVALID_ARGUMENT;
    }
    cudaEventRecord(E.ev0, E.stream);
    TT_TRY(run_range_tt(v, 0, 0, nw, 0, (int)mind, (int)maxd));
    TT_TRY(run_range_tt(v, 0, nw, n - nw, 1, (int)mind, (int)maxd));
    k_tt_finish<<<small_grid(n), 256, 0, E.stream>>>(E.lv[0].v, n, g_tt.lv[0], g_tt.active, g_tt.root_of, d_out,
                                                     g_tt.counters);
    TT_CUDA(cudaGetLastError());
    cudaEventRecord(E.ev1, E.stream);
    u64 c[4];
    TT_CUDA(cudaMemcpyAsync(c, g_tt.counters, sizeof(c), cudaMemcpyDeviceToHost, E.stream));
    TT_CUDA(cudaEventSynchronize(E.ev1));
    TT_CUDA(cudaStreamSynchronize(E.stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, E.ev0, E.ev1);
    E.st.device_ms = ms;
    E.st.tt_probes = c[0];
    E.st.tt_hits = c[1];
    E.st.tt_stores = c[2];
    return PG_OK;
}

}  // namespace pg

// ===========================================================================
// C ABI: host-side key and entry helpers (the same inline code the kernels
// run; no GPU needed)
// ===========================================================================

using namespace pg;

extern "C" {

static const ulonglong2* host_key_table()
{
    static ulonglong2 keys[ZOBRIST_KEYS];
    static const bool made = (zobrist_key_table(keys), true);
    (void)made;
    return keys;
}

int pg_zobrist_key(const pg_board* pos, uint64_t key[2])
{
    if (!pos || !key) {
        set_error("null argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    u64 w[6];
    memcpy(w, pos, sizeof(w));
    const ulonglong2 h = zobrist128(w, host_key_table());
    key[0] = h.x;
    key[1] = h.y;
    return PG_OK;
}

int pg_zobrist_key_from(const pg_board* from, const uint64_t from_key[2], const pg_board* pos, uint64_t key[2])
{
    if (!from || !from_key || !pos || !key) {
        set_error("null argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    u64 pw[6], cw[6];
    memcpy(pw, from, sizeof(pw));
    memcpy(cw, pos, sizeof(cw));
    const ulonglong2 h = zobrist128_from(pw, make_ulonglong2(from_key[0], from_key[1]), cw, host_key_table());
    key[0] = h.x;
    key[1] = h.y;
    return PG_OK;
}

int pg_tt_entry_pack(const uint64_t key[2], uint64_t count, uint64_t entry[4])
{
    if (!key || !entry) {
        set_error("null argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    ulonglong2 a, b;
    tt_pack(key[0], key[1], count, a, b);
    entry[0] = a.x;
    entry[1] = a.y;
    entry[2] = b.x;
    entry[3] = b.y;
    return PG_OK;
}

int pg_tt_entry_match(const uint64_t entry[4], const uint64_t key[2], int* accepted, uint64_t* count)
{
    if (!entry || !key || !accepted) {
        set_error("null argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    u64 v = 0;
    const bool ok = tt_match(make_ulonglong2(entry[0], entry[1]), make_ulonglong2(entry[2], entry[3]), key[0],
                             key[1], v);
    *accepted = ok ? 1 : 0;
    if (count) *count = ok ? v : 0;
    return PG_OK;
}

}  // extern "C"
