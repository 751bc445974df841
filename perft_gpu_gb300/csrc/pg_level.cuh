// pg_level.cuh -- level-buffer access and the table-free kernels of the
// breadth-first driver: root partition, exclusive scan, chunk planning.
#pragma once
#include <cuda/atomic>

#include "pg_engine.cuh"

namespace pg {

// remaining-depth value of a node that needs no further work (a
// transposition-table hit or a duplicate of another node of its level)
constexpr unsigned char REM_DEAD = 0x80;

__device__ __forceinline__ Pos load_board(const LevelView& lv, u64 i)
{
    const ulonglong2 a = lv.pl0[i], b = lv.pl1[i], c = lv.pl2[i];
    return Pos{a.x, a.y, b.x, b.y, c.x, c.y};
}
__device__ __forceinline__ void store_board(const LevelView& lv, u64 i, const Pos& p)
{
    lv.pl0[i] = make_ulonglong2(p.w, p.p);
    lv.pl1[i] = make_ulonglong2(p.n, p.bq);
    lv.pl2[i] = make_ulonglong2(p.rq, p.k);
}

// roots into level 0, white-to-move first, black-to-move from the end
static __global__ void k_partition_roots(const Pos* __restrict__ in, const unsigned char* __restrict__ depths, u32 n,
                                  LevelView lv, u32* counters /* [0] white, [1] black, [2] min depth, [3] max depth */,
                                  const u32* __restrict__ groups = nullptr /* group id per root; null = index */)
{
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Pos b = in[i];
        const u32 d = depths[i];
        u32 slot;
        if (st_side(b)) slot = n - 1 - atomicAdd(&counters[1], 1u);
        else slot = atomicAdd(&counters[0], 1u);
        store_board(lv, slot, b);
        lv.grp[slot] = groups ? groups[i] : i;
        lv.rem[slot] = (unsigned char)d;
        atomicMin(&counters[2], d);
        atomicMax(&counters[3], d);
    }
}

constexpr int SCAN_T = 256;
constexpr int SCAN_V = 8;
constexpr int SCAN_TILE = SCAN_T * SCAN_V;
constexpr u64 SCAN_FLAG_AGG = 1ull << 62;
constexpr u64 SCAN_FLAG_PRE = 2ull << 62;
constexpr u64 SCAN_VAL = (1ull << 62) - 1;
constexpr u32 SCAN_SPIN_LIMIT = 1u << 22;

// exclusive scan of n u32 counts into n+1 u64 offsets (out[n] = total).
// status[] (one word per tile) and *ticket must be zero on entry.
static __global__ void __launch_bounds__(SCAN_T) k_scan(const u32* __restrict__ in, u32 n, u64* __restrict__ out,
                                                 u64* status, u32* ticket, u32* err)
{
    __shared__ u32 s_tile;
    __shared__ u64 s_warp[SCAN_T / 32];
    __shared__ u64 s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const u32 tile = s_tile;
    const u64 base = (u64)tile * SCAN_TILE + (u64)tid * SCAN_V;
    u32 v[SCAN_V];
    u64 tsum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_V; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        tsum += v[k];
    }
    u64 x = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u64 y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        u64 w = lane < SCAN_T / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u64 y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SCAN_T / 32) s_warp[lane] = w;
    }
    __syncthreads();
    const u64 aggregate = s_warp[SCAN_T / 32 - 1];
    const u64 texcl = (warp ? s_warp[warp - 1] : 0ull) + x - tsum;
    if (tid == 0) {
        cuda::atomic_ref<u64, cuda::thread_scope_device> mine(status[tile]);
        if (tile == 0) {
            mine.store(SCAN_FLAG_PRE | aggregate, cuda::memory_order_release);
            s_prefix = 0;
        } else {
            mine.store(SCAN_FLAG_AGG | aggregate, cuda::memory_order_release);
            u64 prefix = 0;
            long j = (long)tile - 1;
            u32 spins = 0;
            while (j >= 0) {
                cuda::atomic_ref<u64, cuda::thread_scope_device> st(status[j]);
                const u64 w = st.load(cuda::memory_order_acquire);
                if ((w & ~SCAN_VAL) == 0) {
                    if (++spins > SCAN_SPIN_LIMIT) {
                        atomicOr(err, ERR_SCAN_TIMEOUT);
                        break;
                    }
                    __nanosleep(32);
                    continue;
                }
                prefix += w & SCAN_VAL;
                if (w & SCAN_FLAG_PRE) break;
                --j;
            }
            mine.store(SCAN_FLAG_PRE | (prefix + aggregate), cuda::memory_order_release);
            s_prefix = prefix;
        }
    }
    __syncthreads();
    u64 run = s_prefix + texcl;
#pragma unroll
    for (int k = 0; k < SCAN_V; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if ((u64)tile * SCAN_TILE + SCAN_TILE >= n && tid == SCAN_T - 1) out[n] = s_prefix + aggregate;
}

// greedy chunking: consecutive node ranges whose children fit `cap`
static __global__ void k_plan(const u64* __restrict__ offs, u32 n, u64 cap, PlanOut* plan, u32* err)
{
    if (threadIdx.x || blockIdx.x) return;
    u32 a = 0, k = 0;
    plan->bnd[0] = 0;
    plan->coff[0] = offs[0];
    while (a < n && k < MAX_CHUNKS) {
        const u64 limit = offs[a] + cap;
        u32 lo = a + 1, hi = n;  // largest b in [a+1, n] with offs[b] <= limit
        if (offs[lo] > limit) {
            hi = lo;  // one node alone exceeds the cap; cannot happen for cap >= 256
            atomicOr(err, ERR_PLAN_OVERFLOW);
        }
        while (lo < hi) {
            const u32 mid = lo + (hi - lo + 1) / 2;
            if (offs[mid] <= limit) lo = mid; else hi = mid - 1;
        }
        plan->bnd[++k] = lo;
        plan->coff[k] = offs[lo];
        a = lo;
    }
    if (a < n) atomicOr(err, ERR_PLAN_OVERFLOW);
    plan->nchunks = k;
    plan->total = offs[n];
}

// largest depth of a batch (out zeroed by the caller)
static __global__ void k_max_depth(const unsigned char* __restrict__ dep, u32 n, u32* out)
{
    u32 m = 0;
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = max(m, (u32)dep[i]);
    m = __reduce_max_sync(0xFFFFFFFFu, m);
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// order-sensitive 64-bit checksum of a batch (boards and depths)
static __global__ void k_checksum(const Pos* __restrict__ pos, const unsigned char* __restrict__ dep, u32 n, u64* out)
{
    u64 h = 0;
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Pos b = pos[i];
        u64 x = (u64)i * 0x9E3779B97F4A7C15ull + dep[i];
        const u64 w[6] = {b.w, b.p, b.n, b.bq, b.rq, b.k};
#pragma unroll
        for (int k = 0; k < 6; k++) {
            x ^= w[k] + 0x632BE59BD9B4E019ull * (k + 1);
            x *= 0xD6E8FEB86659FD93ull;
            x ^= x >> 32;
        }
        h ^= x;
    }
    for (int o = 16; o; o >>= 1) h ^= __shfl_xor_sync(0xFFFFFFFFu, h, o);
    if ((threadIdx.x & 31) == 0 && h) atomicXor(out, h);
}

// level nodes [0, n) of one level buffer into an array of boards
static __global__ void k_level_to_boards(LevelView lv, u32 n, Pos* __restrict__ out)
{
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = load_board(lv, i);
}

}  // namespace pg
