// pg_kernels.cuh -- CUDA kernels of the perft engine (sm_103a).
//
// Breadth-first expansion of the reference's GPU path (perft_bb.h:1027-1138:
// per level count -> exclusive scan -> parent expansion -> generate + make,
// count-only leaf) re-planned for one GB300:
//   k_count_level   children per node of a level (countMoves)
//   k_scan          single-pass exclusive scan, decoupled look-back with a
//                   bounded spin (replaces moderngpu ScanD, scan.cuh:330)
//   k_plan          greedy split of a level into chunks whose children fit
//                   the next level's buffer (HBM budget)
//   k_expand        generate + make into the next level; the CTA stages its
//                   nodes in shared memory, emits (parent, move) entries into
//                   a shared queue and writes children coalesced in 16-byte
//                   vectors (replaces IntervalExpand + generate_moves +
//                   makemove_and_count, perft_bb.h:601,983; intervalmove.cuh:405)
//   k_leaf          the last two plies inside one CTA: count each node's
//                   moves, scan in shared memory, queue (parent, move)
//                   entries, then every thread makes + counts entries, so
//                   the per-thread work is even whatever the branching
//                   (replaces makeMove_and_perft_single_level_indices,
//                   perft_bb.h:412)
#pragma once
#include "pg_level.cuh"
#include "pg_movegen.cuh"

namespace pg {

// per-thread running sum for one group id; flushed with one atomic per
// group change and one per warp at the end when the warp shares the group
struct GroupAcc {
    static constexpr u32 NONE = 0xFFFFFFFFu;
    u32 g = NONE;
    u64 s = 0;
    __device__ __forceinline__ void add(u64* acc, u32 grp, u64 v)
    {
        if (grp != g) {
            if (s) atomicAdd(&acc[g], s);
            g = grp;
            s = 0;
        }
        s += v;
    }
    __device__ __forceinline__ void flush_warp(u64* acc)
    {
        const unsigned full = 0xFFFFFFFFu;
        const u32 g0 = __shfl_sync(full, g, 0);
        const bool same = __all_sync(full, g == g0 || s == 0);
        if (same) {
            u64 t = s;
            for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(full, t, o);
            if ((threadIdx.x & 31) == 0 && t && g0 != NONE) atomicAdd(&acc[g0], t);
        } else if (s) {
            atomicAdd(&acc[g], s);
        }
        s = 0;
        g = NONE;
    }
};

// exclusive scan of one u32 per thread over a CTA of T threads
template <int T>
__device__ __forceinline__ u32 block_excl_scan(u32 v, u32& total, u32* s_warp)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u32 x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u32 y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        u32 w = lane < T / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < T / 32) s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[T / 32 - 1];
    return (warp ? s_warp[warp - 1] : 0u) + x - v;
}

// writes the moves of one node whose queue positions fall in [lo, hi)
struct QEmit {
    u32* q;
    u32 pos, lo, hi, tag;
    __device__ __forceinline__ void operator()(u16 m)
    {
        if (pos >= lo && pos < hi) q[pos - lo] = tag | m;
        ++pos;
    }
    // bits 25-28 carry the moving piece (PC_*) and PC_EP_FLAG for make_child
    __device__ __forceinline__ void operator()(u16 m, u32 piece)
    {
        if (pos >= lo && pos < hi) q[pos - lo] = tag | m | (piece << 25);
        ++pos;
    }
};

// QEmit when every move of the CTA's nodes fits the queue (one window)
struct QEmitAll {
    u32* q;
    u32 pos, tag;
    __device__ __forceinline__ void operator()(u16 m) { q[pos++] = tag | m; }
    __device__ __forceinline__ void operator()(u16 m, u32 piece) { q[pos++] = tag | m | (piece << 25); }
};

struct ArrEmit {
    u16* out;
    u32 n;
    __device__ __forceinline__ void operator()(u16 m)
    {
        if (n < 256) out[n] = m;
        ++n;
    }
};

struct BoardEmit {
    Pos* out;
    u32 n;
    __device__ __forceinline__ void operator()(const Pos& p)
    {
        if (n < 256) out[n] = p;
        ++n;
    }
};

template <class SL> __device__ __forceinline__ u32 count_any(const Pos& b)
{
    return st_side(b) ? count_moves<1, SL>(b) : count_moves<0, SL>(b);
}

// ---------------------------------------------------------------------------
// operator-surface kernels (mixed sides, one thread per position)
// ---------------------------------------------------------------------------

template <class SL>
__global__ void k_count_batch(const Pos* __restrict__ in, u32 n, u32* __restrict__ out)
{
    stage_tables<SL>();
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = count_any<SL>(in[i]);
}

template <class SL>
__global__ void k_gen_moves_batch(const Pos* __restrict__ in, u32 n, u16* __restrict__ out, u32* __restrict__ nout)
{
    stage_tables<SL>();
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        ArrEmit e{out + (u64)i * 256, 0};
        const Pos b = in[i];
        if (st_side(b)) gen_moves<1, SL>(b, e); else gen_moves<0, SL>(b, e);
        nout[i] = e.n;
    }
}

template <class SL>
__global__ void k_gen_boards_batch(const Pos* __restrict__ in, u32 n, Pos* __restrict__ out, u32* __restrict__ nout)
{
    stage_tables<SL>();
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        BoardEmit e{out + (u64)i * 256, 0};
        const Pos b = in[i];
        if (st_side(b)) gen_boards<1, SL>(b, e); else gen_boards<0, SL>(b, e);
        nout[i] = e.n;
    }
}

static __global__ void k_make_batch(Pos* __restrict__ pos, const u16* __restrict__ mv, u32 n)
{
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        Pos b = pos[i];
        if (st_side(b)) make_move<1>(b, mv[i]); else make_move<0>(b, mv[i]);
        pos[i] = b;
    }
}

__device__ __forceinline__ u64 splitmix_next(u64& s)
{
    u64 z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// seeded random legal playouts (procedure documented at pg_random_playouts)
template <class SL>
__global__ void k_playouts(Pos start, u64 seed, u32 n, int min_plies, int max_plies, int min_moves, int depth_lo,
                           int depth_hi, Pos* __restrict__ out, unsigned char* __restrict__ depths, u32* err)
{
    stage_tables<SL>();
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        u16 mv[256];
        bool done = false;
        for (u64 a = 0; a < 100000 && !done; a++) {
            u64 s = seed ^ ((u64)i << 32) ^ (a * 0xA24BAED4963EE407ull);
            const int plies = min_plies + (int)(splitmix_next(s) % (u64)(max_plies - min_plies + 1));
            Pos p = start;
            bool ok = true;
            for (int k = 0; k < plies; k++) {
                ArrEmit e{mv, 0};
                if (st_side(p)) gen_moves<1, SL>(p, e); else gen_moves<0, SL>(p, e);
                if (!e.n) {
                    ok = false;
                    break;
                }
                const u16 m = mv[splitmix_next(s) % min(e.n, 256u)];
                if (st_side(p)) make_move<1>(p, m); else make_move<0>(p, m);
            }
            if (ok && (int)count_any<SL>(p) >= min_moves) {
                out[i] = p;
                done = true;
            }
        }
        if (!done) atomicOr(err, ERR_PLAYOUT_ATTEMPTS);
        if (depths) {
            u64 s = seed ^ ((u64)i << 32) ^ 0x5851F42D4C957F2Dull;
            depths[i] = (unsigned char)(depth_lo + (int)(splitmix_next(s) % (u64)(depth_hi - depth_lo + 1)));
        }
    }
}

// ---------------------------------------------------------------------------
// engine kernels
// ---------------------------------------------------------------------------

// The bodies of the level kernels are device functions so that the
// persistent driver (pg_persist.cuh) runs the same code as the per-level
// launches; the kernels below are thin wrappers.  The bodies take no
// __restrict__ on data another phase of a persistent launch writes.

template <int S, class SL>
__device__ __forceinline__ void count_level_body(const LevelView& lv, u32 start, u32 n, u32* cnt, u32 min_rem)
{
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const u32 rem = lv.rem[start + i];
        cnt[i] = (rem >= min_rem && rem < REM_DEAD) ? count_moves<S, SL>(load_board(lv, start + i)) : 0u;
    }
}

template <int S, class SL>
__global__ void k_count_level(LevelView lv, u32 start, u32 n, u32* __restrict__ cnt, u32 min_rem)
{
    stage_tables<SL>();
    count_level_body<S, SL>(lv, start, n, cnt, min_rem);
}

template <class SL, int T, int QCAP> struct BlockSmem {
    static constexpr int tables = table_smem_bytes<SL>();
    static constexpr int boards = T * (int)sizeof(Pos);
    static constexpr int queue = QCAP * 4;
    static constexpr int bytes = tables + boards + queue + T * 4 + T;
};

// register cap: at least PG_LEAF_MIN_WARPS resident warps per SM
#ifndef PG_LEAF_MIN_WARPS
#define PG_LEAF_MIN_WARPS 16
#endif
template <int T> constexpr int min_blocks() { return (PG_LEAF_MIN_WARPS * 32 + T - 1) / T; }

// the last plies of every node with remaining depth <= 2, inside one CTA
// (pg_leaf_body.inc).  The kernel includes the statements in its own body,
// not through this function: with the arguments left in the parameter space
// the compiler keeps more registers for the count (measured 0.5-0.9% faster
// than calling the inlined function).  LV is LevelView or any type with the
// same grp[] / rem[] subscripts and a load_board overload.
template <int S, class SL, int T, int QCAP, class LV>
__device__ __forceinline__ void leaf_body(LV lv, u32 start, u32 n, u64* __restrict__ acc, u32* ticket, u32 max_rem)
{
    extern __shared__ __align__(16) unsigned char pg_dyn_smem[];
#include "pg_leaf_body.inc"
}

template <int S, class SL, int T, int QCAP>
__global__ void __launch_bounds__(T, min_blocks<T>()) k_leaf(LevelView lv, u32 start, u32 n, u64* __restrict__ acc, u32* ticket,
                                                            u32 max_rem)
{
    extern __shared__ __align__(16) unsigned char pg_dyn_smem[];
    stage_tables<SL>();
#include "pg_leaf_body.inc"
}

// children of the nodes [a, b) of a level into the next level; offs is the
// exclusive scan of the children counts, child slots start at offs[a]
// parent_out (transposition-table mode): each child's group becomes its own
// slot and its parent's slot is written to parent_out
template <int S, class SL, int T, int QCAP>
__device__ __forceinline__ void expand_body(const LevelView& in, u32 start, u32 a, u32 b, const u64* offs,
                                            const LevelView& out, u32* ticket, u32* parent_out)
{
    extern __shared__ __align__(16) unsigned char pg_dyn_smem[];
    using L = BlockSmem<SL, T, QCAP>;
    Pos* sb = reinterpret_cast<Pos*>(pg_dyn_smem + L::tables);
    u32* q = reinterpret_cast<u32*>(pg_dyn_smem + L::tables + L::boards);
    u32* sg = q + QCAP;
    unsigned char* sr = reinterpret_cast<unsigned char*>(sg + T);
    __shared__ u32 s_chunk;
    const int tid = threadIdx.x;
    const u64 out_base = offs[a];
    for (;;) {
        if (tid == 0) s_chunk = atomicAdd(ticket, 1u);
        __syncthreads();
        const u64 c0 = (u64)a + (u64)s_chunk * T;
        if (c0 >= b) break;
        const u64 c1 = min(c0 + T, (u64)b);
        const u64 i = c0 + tid;
        const u64 chunk_off = offs[c0];
        const u32 total = (u32)(offs[c1] - chunk_off);
        const u64 chunk_out = chunk_off - out_base;
        Pos bd{0, 0, 0, 0, 0, 0};
        u32 c = 0, off = 0;
        if (i < c1) {
            const u64 o0 = offs[i];
            c = (u32)(offs[i + 1] - o0);
            off = (u32)(o0 - chunk_off);
            bd = load_board(in, start + i);
            sg[tid] = in.grp[start + i];
            sr[tid] = in.rem[start + i];
        }
        sb[tid] = bd;
        for (u32 lo = 0; lo < total; lo += QCAP) {
            const u32 hi = min(lo + (u32)QCAP, total);
            if (c && off < hi && off + c > lo) {
                QEmit e{q, off, lo, hi, (u32)tid << 16};
                gen_leaf<S>(bd, e);
            }
            __syncthreads();
            const u32 m = hi - lo;
            for (u32 e = tid; e < m; e += T) {
                const u32 ent = q[e];
                const u32 p = (ent >> 16) & (T - 1);  // in bounds even if a queue slot was left unwritten
                Pos ch = sb[p];
                make_move<S>(ch, (u16)(ent & 0xFFFFu));
                const u64 o = chunk_out + lo + e;
                store_board(out, o, ch);
                if (parent_out) {
                    out.grp[o] = (u32)o;
                    parent_out[o] = (u32)(start + c0 + p);
                } else {
                    out.grp[o] = sg[p];
                }
                out.rem[o] = (unsigned char)(sr[p] - 1);
            }
            __syncthreads();
        }
        __syncthreads();
    }
}

template <int S, class SL, int T, int QCAP>
__global__ void __launch_bounds__(T, min_blocks<T>()) k_expand(LevelView in, u32 start, u32 a, u32 b, const u64* __restrict__ offs,
                                              LevelView out, u32* ticket, u32* __restrict__ parent_out = nullptr)
{
    stage_tables<SL>();
    expand_body<S, SL, T, QCAP>(in, start, a, b, offs, out, ticket, parent_out);
}

}  // namespace pg
