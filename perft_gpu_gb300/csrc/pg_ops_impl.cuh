// pg_ops_impl.cuh -- launch wrappers instantiated once per slider policy.
// Included by exactly one translation unit per policy (pg_sl_*.cu).
#pragma once
#include <algorithm>

#include "pg_kernels.cuh"
#include "pg_ops.cuh"

namespace pg {
namespace {

// shared-memory queue entries per CTA: 64 per thread hold the children of
// a CTA's nodes in one window even for positions with ~50 moves (the leaf
// kernel's first window generates from the count's analysis; a second
// window makes it again and runs a second copy of the hot loop); the
// byte-lookup policy gives 158 KB of the CTA's shared memory to its tables
// and keeps 8
template <class SL, int T> struct QcapFor {
    static constexpr int value = SL::kId == 2 ? T * 8 : T * 64;
};

inline int occupancy_grid(const void* fn, int T, int smem, u64 items, int num_sms)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, T, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const u64 want = std::max<u64>(1, (items + T - 1) / T);
    return (int)std::min<u64>(want, (u64)per_sm * (u64)num_sms);
}

template <class SL>
cudaError_t upload_tables(const HostTables& t)
{
    return upload_static_tables(t);
}

template <class K> cudaError_t set_smem(K fn, int bytes)
{
    return bytes > 48 * 1024 ? cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)
                             : cudaSuccess;
}

template <int S, class SL, int T>
cudaError_t leaf_t(const LevelView& lv, u32 start, u32 n, u64* acc, u32* ticket, u32 max_rem, cudaStream_t st,
                   int sms)
{
    constexpr int Q = QcapFor<SL, T>::value;
    using L = BlockSmem<SL, T, Q>;
    auto fn = k_leaf<S, SL, T, Q>;
    static cudaError_t attr = set_smem(fn, L::bytes);
    if (attr) return attr;
    const int grid = occupancy_grid((const void*)fn, T, L::bytes, n, sms);
    fn<<<grid, T, L::bytes, st>>>(lv, start, n, acc, ticket, max_rem);
    return cudaGetLastError();
}

template <int S, class SL, int T>
cudaError_t expand_t(const LevelView& in, u32 start, u32 a, u32 b, const u64* offs, const LevelView& out, u32* ticket,
                     cudaStream_t st, int sms)
{
    constexpr int Q = QcapFor<SL, T>::value;
    using L = BlockSmem<SL, T, Q>;
    auto fn = k_expand<S, SL, T, Q>;
    static cudaError_t attr = set_smem(fn, L::bytes);
    if (attr) return attr;
    const int grid = occupancy_grid((const void*)fn, T, L::bytes, (u64)(b - a), sms);
    fn<<<grid, T, L::bytes, st>>>(in, start, a, b, offs, out, ticket, nullptr);
    return cudaGetLastError();
}

template <class SL>
cudaError_t leaf_any(int side, int T, const LevelView& lv, u32 start, u32 n, u64* acc, u32* ticket, u32 max_rem,
                     cudaStream_t st, int sms)
{
    if (T == 128)
        return side ? leaf_t<1, SL, 128>(lv, start, n, acc, ticket, max_rem, st, sms)
                    : leaf_t<0, SL, 128>(lv, start, n, acc, ticket, max_rem, st, sms);
    if (T == 512)
        return side ? leaf_t<1, SL, 512>(lv, start, n, acc, ticket, max_rem, st, sms)
                    : leaf_t<0, SL, 512>(lv, start, n, acc, ticket, max_rem, st, sms);
    return side ? leaf_t<1, SL, 256>(lv, start, n, acc, ticket, max_rem, st, sms)
                : leaf_t<0, SL, 256>(lv, start, n, acc, ticket, max_rem, st, sms);
}

template <class SL>
cudaError_t expand_any(int side, int T, const LevelView& in, u32 start, u32 a, u32 b, const u64* offs,
                       const LevelView& out, u32* ticket, cudaStream_t st, int sms)
{
    if (T == 128) return side ? expand_t<1, SL, 128>(in, start, a, b, offs, out, ticket, st, sms) : expand_t<0, SL, 128>(in, start, a, b, offs, out, ticket, st, sms);
    if (T == 512) return side ? expand_t<1, SL, 512>(in, start, a, b, offs, out, ticket, st, sms) : expand_t<0, SL, 512>(in, start, a, b, offs, out, ticket, st, sms);
    return side ? expand_t<1, SL, 256>(in, start, a, b, offs, out, ticket, st, sms) : expand_t<0, SL, 256>(in, start, a, b, offs, out, ticket, st, sms);
}

template <int S, class SL>
cudaError_t count_level_t(const LevelView& lv, u32 start, u32 n, u32* cnt, u32 min_rem, cudaStream_t st, int sms)
{
    auto fn = k_count_level<S, SL>;
    constexpr int smem = table_smem_bytes<SL>();
    static cudaError_t attr = set_smem(fn, smem);
    if (attr) return attr;
    const int grid = occupancy_grid((const void*)fn, 256, smem, n, sms);
    fn<<<grid, 256, smem, st>>>(lv, start, n, cnt, min_rem);
    return cudaGetLastError();
}

template <class SL>
cudaError_t count_level_any(int side, const LevelView& lv, u32 start, u32 n, u32* cnt, u32 min_rem, cudaStream_t st,
                            int sms)
{
    return side ? count_level_t<1, SL>(lv, start, n, cnt, min_rem, st, sms)
                : count_level_t<0, SL>(lv, start, n, cnt, min_rem, st, sms);
}

inline int small_grid(u32 n, int T) { return (int)std::max<u32>(1, std::min<u32>((n + T - 1) / T, 8192)); }

template <class SL>
cudaError_t count_batch(const Pos* in, u32 n, u32* out, cudaStream_t st)
{
    constexpr int smem = table_smem_bytes<SL>();
    static cudaError_t attr = set_smem(k_count_batch<SL>, smem);
    if (attr) return attr;
    k_count_batch<SL><<<small_grid(n, 128), 128, smem, st>>>(in, n, out);
    return cudaGetLastError();
}

template <class SL>
cudaError_t gen_moves_batch(const Pos* in, u32 n, u16* out, u32* nout, cudaStream_t st)
{
    constexpr int smem = table_smem_bytes<SL>();
    static cudaError_t attr = set_smem(k_gen_moves_batch<SL>, smem);
    if (attr) return attr;
    k_gen_moves_batch<SL><<<small_grid(n, 128), 128, smem, st>>>(in, n, out, nout);
    return cudaGetLastError();
}

template <class SL>
cudaError_t gen_boards_batch(const Pos* in, u32 n, Pos* out, u32* nout, cudaStream_t st)
{
    constexpr int smem = table_smem_bytes<SL>();
    static cudaError_t attr = set_smem(k_gen_boards_batch<SL>, smem);
    if (attr) return attr;
    k_gen_boards_batch<SL><<<small_grid(n, 128), 128, smem, st>>>(in, n, out, nout);
    return cudaGetLastError();
}

inline cudaError_t make_batch(Pos* pos, const u16* mv, u32 n, cudaStream_t st)
{
    k_make_batch<<<small_grid(n, 128), 128, 0, st>>>(pos, mv, n);
    return cudaGetLastError();
}

template <class SL>
cudaError_t playouts(const Pos& start, u64 seed, u32 n, int min_plies, int max_plies, int min_moves, int depth_lo,
                     int depth_hi, Pos* out, unsigned char* depths, u32* err, cudaStream_t st)
{
    constexpr int smem = table_smem_bytes<SL>();
    static cudaError_t attr = set_smem(k_playouts<SL>, smem);
    if (attr) return attr;
    k_playouts<SL><<<small_grid(n, 64), 64, smem, st>>>(start, seed, n, min_plies, max_plies, min_moves, depth_lo,
                                                          depth_hi, out, depths, err);
    return cudaGetLastError();
}

}  // namespace

#define PG_DEFINE_OPS(SLT, NAME, ENUM)                                                                   \
    const SliderOps g_ops_##NAME = {#NAME,          ENUM,                    upload_tables<SLT>,           \
                                    leaf_any<SLT>,  expand_any<SLT>,         count_level_any<SLT>,         \
                                    count_batch<SLT>, gen_moves_batch<SLT>,  gen_boards_batch<SLT>,        \
                                    make_batch,     playouts<SLT>};

}  // namespace pg
