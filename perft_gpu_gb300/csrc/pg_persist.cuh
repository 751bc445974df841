// pg_persist.cuh -- the whole chunked breadth-first perft of a batch in one
// persistent, cooperative launch.
//
// The per-level driver (run_range, pg_engine.cu) launches count, scan, plan,
// expand and leaf kernels level by level and reads every level's chunk plan
// back to the host.  Here one kernel with every CTA resident (cooperative
// launch: one CTA per free slot of every SM) walks the same recursion on the
// device: all CTAs run the same control loop over an explicit stack of
// (level, range, side, remaining-depth bounds, chunk) frames, decide from
// data in global memory that a grid barrier made visible, and execute each
// phase together -- root partition, leaf (the last two plies inside a CTA),
// children count, decoupled look-back scan, chunk plan (one thread), expand
// into the next level.  Load balancing inside a phase is the CTA-queue
// tickets of the leaf and expand bodies; between phases a grid barrier.  The
// host issues one launch per call and reads nothing back until it ends, so a
// batch is one kernel in a CUDA graph whatever its contents.
//
// Every wait is bounded: a CTA waiting at a grid barrier gives up after
// PERSIST_BARRIER_NS of global time, sets ERR_GRID_BARRIER_TIMEOUT and an
// abort word that every CTA checks while it waits and after each barrier, so
// the launch ends with an error the host reads instead of hanging; the
// scan's look-back keeps its poll limit (ERR_SCAN_TIMEOUT).  A level deeper
// than the buffers the host prepared sets ERR_LEVEL_CAP, more phases than
// tickets or a chunk plan that cannot be made ERR_PLAN_OVERFLOW, and the
// launch ends.
//
// The reference's counterpart is its device-side driver
// (perft_bb_gpu_simple, perft_bb.h:1027-1138, launched through dynamic
// parallelism from perft_bb_driver_gpu, perft_bb.h:1143-1220).
#pragma once
#include <cuda/atomic>

#include "pg_kernels.cuh"

namespace pg {

constexpr u64 PERSIST_BARRIER_NS = 60ull * 1000 * 1000 * 1000;  // 60 s of global time per barrier
constexpr int PERSIST_T = PERSIST_CTA;
constexpr int PERSIST_Q = PERSIST_T * 64;                        // queue entries per CTA (as k_leaf)
constexpr int PERSIST_SCAN_V = 8;                                // counts per thread per scan tile
constexpr int PERSIST_SCAN_TILE = PERSIST_T * PERSIST_SCAN_V;
static_assert(PERSIST_SCAN_TILE == (int)PERSIST_SCAN_TILE_NODES, "scan tile known to the host");

// ends the launch with an error: every other CTA leaves at its next barrier
__device__ __forceinline__ void persist_fail(const PersistArgs& A, u32 bit)
{
    atomicOr(A.err, bit);
    cuda::atomic_ref<u32, cuda::thread_scope_device>(A.ctl->abort).store(1u, cuda::memory_order_relaxed);
}

__device__ __forceinline__ u64 global_ns()
{
    u64 t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// grid-wide barrier of a cooperative launch; false when the launch is being
// abandoned (a barrier gave up, or another CTA raised the abort word)
__device__ __forceinline__ bool grid_barrier(PersistCtl* ctl, u32* err)
{
    __shared__ u32 s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        u32 ok = 1;
        cuda::atomic_ref<u32, cuda::thread_scope_device> count(ctl->bar_count), gen(ctl->bar_gen),
            abort(ctl->abort);
        const u32 g = gen.load(cuda::memory_order_relaxed);
        __threadfence();  // this CTA's writes before its arrival
        if (count.fetch_add(1u, cuda::memory_order_acq_rel) == gridDim.x - 1) {
            count.store(0u, cuda::memory_order_relaxed);
            gen.store(g + 1u, cuda::memory_order_release);
        } else {
            const u64 t0 = global_ns();
            u32 polls = 0;
            while (gen.load(cuda::memory_order_acquire) == g) {
                if (abort.load(cuda::memory_order_relaxed)) break;
                if ((++polls & 255u) == 0 && global_ns() - t0 > PERSIST_BARRIER_NS) {
                    atomicOr(err, ERR_GRID_BARRIER_TIMEOUT);
                    abort.store(1u, cuda::memory_order_relaxed);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();  // the other CTAs' writes before this CTA reads on
        if (abort.load(cuda::memory_order_relaxed)) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// exclusive scan of n counts into n + 1 offsets (out[n] = total) by the CTAs
// of the launch: tiles in ticket order, decoupled look-back (a predecessor's
// tile is always held by a resident CTA); status[] zero on entry
__device__ __forceinline__ void persist_scan(const u32* in, u32 n, u64* out, u64* status, u32* ticket, u32* err)
{
    constexpr int T = PERSIST_T, V = PERSIST_SCAN_V;
    __shared__ u32 s_tile;
    __shared__ u64 s_warp[T / 32];
    __shared__ u64 s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const u32 ntiles = (n + PERSIST_SCAN_TILE - 1) / PERSIST_SCAN_TILE;
    if (n == 0) {
        if (blockIdx.x == 0 && tid == 0) out[0] = 0;
        return;
    }
    for (;;) {
        __syncthreads();  // s_tile of the previous tile has been read
        if (tid == 0) s_tile = atomicAdd(ticket, 1u);
        __syncthreads();
        const u32 tile = s_tile;
        if (tile >= ntiles) break;
        const u64 base = (u64)tile * PERSIST_SCAN_TILE + (u64)tid * V;
        u32 v[V];
        u64 tsum = 0;
#pragma unroll
        for (int k = 0; k < V; k++) {
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
            u64 w = lane < T / 32 ? s_warp[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const u64 y = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if (lane >= o) w += y;
            }
            if (lane < T / 32) s_warp[lane] = w;
        }
        __syncthreads();
        const u64 aggregate = s_warp[T / 32 - 1];
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
        for (int k = 0; k < V; k++) {
            if (base + k < n) out[base + k] = run;
            run += v[k];
        }
        if (tile == ntiles - 1 && tid == T - 1) out[n] = s_prefix + aggregate;
    }
}

// greedy chunks of nodes [0, n) whose children fit cap (one thread)
__device__ __forceinline__ void persist_plan(const u64* offs, u32 n, u64 cap, PlanOut* plan, u32* err)
{
    u32 a = 0, k = 0;
    plan->bnd[0] = 0;
    plan->coff[0] = offs[0];
    while (a < n && k < MAX_CHUNKS) {
        const u64 limit = offs[a] + cap;
        u32 lo = a + 1, hi = n;  // largest b in [a+1, n] with offs[b] <= limit
        if (offs[lo] > limit) {
            hi = lo;  // one node alone exceeds the cap (caps are >= 65,536 > 256 moves)
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

// the phases are inlined into the kernel: as called functions the leaf phase
// ran 4-5% slower than k_leaf (measured), inlined about 1%
template <int S>
__device__ __forceinline__ void persist_leaf(const PersistArgs& A, int L, u32 start, u32 n, u32* ticket)
{
    leaf_body<S, SlKS, PERSIST_T, PERSIST_Q>(A.lv[L], start, n, A.acc, ticket, 2u);
}

template <int S>
__device__ __forceinline__ void persist_expand(const PersistArgs& A, int L, u32 start, u32 a, u32 b, u32* ticket)
{
    expand_body<S, SlKS, PERSIST_T, PERSIST_Q>(A.lv[L], start, a, b, A.offs[L], A.lv[L + 1], ticket, nullptr);
}

template <int S>
__device__ __forceinline__ void persist_count(const PersistArgs& A, int L, u32 start, u32 n)
{
    count_level_body<S, SlKS>(A.lv[L], start, n, A.cnt[L], 3u);
}

struct PersistFrame {
    u32 start, n;
    int side, minrem, maxrem;
    u32 k;  // next chunk; 0xFFFFFFFF before the level's own phases ran
};

// One launch: the perft of A.n roots (each root's count added to
// A.acc[group]), two-ply leaf, Kogge-Stone sliders, PERSIST_T threads.
__global__ void __launch_bounds__(PERSIST_T, min_blocks<PERSIST_T>()) k_persist(PersistArgs A)
{
    PersistCtl* ctl = A.ctl;
    // phase 0: roots into level 0, white-to-move first (k_partition_roots)
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        const Pos b = A.pos[i];
        const u32 d = A.depths[i];
        u32 slot;
        if (st_side(b)) slot = A.n - 1 - atomicAdd(&ctl->part[1], 1u);
        else slot = atomicAdd(&ctl->part[0], 1u);
        store_board(A.lv[0], slot, b);
        A.lv[0].grp[slot] = A.groups ? A.groups[i] : i;
        A.lv[0].rem[slot] = (unsigned char)d;
        atomicMin(&ctl->part[2], d);
        atomicMax(&ctl->part[3], d);
    }
    if (!grid_barrier(ctl, A.err)) return;
    using ARef = cuda::atomic_ref<u32, cuda::thread_scope_device>;
    const u32 nw = ARef(ctl->part[0]).load(cuda::memory_order_relaxed);
    const int mind = (int)ARef(ctl->part[2]).load(cuda::memory_order_relaxed);
    const int maxd = (int)ARef(ctl->part[3]).load(cuda::memory_order_relaxed);
    if (maxd > 15) {
        if (blockIdx.x == 0 && threadIdx.x == 0) persist_fail(A, ERR_PLAN_OVERFLOW);
        return;
    }
    u32 tk = 0;  // next ticket: every CTA counts the same phases
    auto ticket = [&]() -> u32* {
        if (tk >= A.max_tickets) return nullptr;
        return A.tickets + tk++;
    };
    PersistFrame stack[MAX_LEVELS];
    for (int side0 = 0; side0 < 2; side0++) {
        const u32 n0 = side0 ? A.n - nw : nw;
        if (n0 == 0) continue;
        int top = 0;
        stack[0] = PersistFrame{side0 ? nw : 0u, n0, side0, mind, maxd, 0xFFFFFFFFu};
        while (top >= 0) {
            PersistFrame& f = stack[top];
            const int L = top;
            if (f.k == 0xFFFFFFFFu) {
                // the level's own phases: leaf, count, scan, plan
                if (f.minrem <= 2) {
                    u32* t = ticket();
                    if (!t) {
                        if (blockIdx.x == 0 && threadIdx.x == 0) persist_fail(A, ERR_PLAN_OVERFLOW);
                        return;
                    }
                    if (f.side) persist_leaf<1>(A, L, f.start, f.n, t);
                    else persist_leaf<0>(A, L, f.start, f.n, t);
                }
                if (f.maxrem <= 2) {
                    --top;
                    continue;
                }
                if (L + 1 >= MAX_LEVELS || A.cap[L + 1] == 0) {
                    if (blockIdx.x == 0 && threadIdx.x == 0) persist_fail(A, ERR_LEVEL_CAP);
                    return;
                }
                if (f.side) persist_count<1>(A, L, f.start, f.n);
                else persist_count<0>(A, L, f.start, f.n);
                const u64 words = (u64)f.n / PERSIST_SCAN_TILE + 2;
                for (u64 i = blockIdx.x * blockDim.x + threadIdx.x; i < words && i < A.status_cap;
                     i += gridDim.x * blockDim.x)
                    A.status[i] = 0;
                if (!grid_barrier(ctl, A.err)) return;
                u32* t = ticket();
                if (!t) {
                    if (blockIdx.x == 0 && threadIdx.x == 0) persist_fail(A, ERR_PLAN_OVERFLOW);
                    return;
                }
                persist_scan(A.cnt[L], f.n, A.offs[L], A.status, t, A.err);
                if (!grid_barrier(ctl, A.err)) return;
                if (blockIdx.x == 0 && threadIdx.x == 0) {
                    persist_plan(A.offs[L], f.n, A.cap[L + 1], A.plan + L, A.err);
                    // a failed scan or plan ends the launch at the barrier below
                    if (*(volatile u32*)A.err) persist_fail(A, 0u);
                }
                if (!grid_barrier(ctl, A.err)) return;
                f.k = 0;
            }
            // the next chunk with children: expand it into level L + 1 and descend
            const PlanOut* pl = A.plan + L;
            const u32 nchunks = pl->nchunks;
            bool descended = false;
            while (f.k < nchunks) {
                const u32 k = f.k++;
                const u32 a = pl->bnd[k], b = pl->bnd[k + 1];
                const u64 children = pl->coff[k + 1] - pl->coff[k];
                if (!children) continue;
                // level L + 1 is free: the previous chunk's subtree has finished
                if (!grid_barrier(ctl, A.err)) return;
                u32* t = ticket();
                if (!t) {
                    if (blockIdx.x == 0 && threadIdx.x == 0) persist_fail(A, ERR_PLAN_OVERFLOW);
                    return;
                }
                if (f.side) persist_expand<1>(A, L, f.start, a, b, t);
                else persist_expand<0>(A, L, f.start, a, b, t);
                if (!grid_barrier(ctl, A.err)) return;
                stack[top + 1] = PersistFrame{0u, (u32)children, 1 - f.side, max(f.minrem, 3) - 1, f.maxrem - 1,
                                              0xFFFFFFFFu};
                ++top;
                descended = true;
                break;
            }
            if (!descended) --top;
        }
        // the other side's roots start at level 0 again: level 1 is reused
        if (!grid_barrier(ctl, A.err)) return;
    }
}

// one CTA per free slot of every SM: all resident, as the barriers need
inline cudaError_t persist_launch_impl(const PersistArgs& a, cudaStream_t st, int num_sms, int* grid)
{
    constexpr int smem = BlockSmem<SlKS, PERSIST_T, PERSIST_Q>::bytes;
    static_assert(smem <= 48 * 1024, "dynamic shared memory above the default limit");
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persist, PERSIST_T, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorLaunchOutOfResources;
    *grid = per_sm * num_sms;
    PersistArgs copy = a;
    void* args[] = {&copy};
    return cudaLaunchCooperativeKernel((const void*)k_persist, dim3(*grid), dim3(PERSIST_T), args, smem, st);
}

}  // namespace pg
