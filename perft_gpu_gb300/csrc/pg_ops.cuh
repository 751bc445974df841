// pg_ops.cuh -- per-slider-policy entry points.  Each policy is compiled in
// its own translation unit (pg_sl_*.cu) with its own copy of the device
// tables; the host driver reaches its kernels through this table.
#pragma once
#include <cuda_runtime.h>

#include "pg_engine.cuh"
#include "pg_tables.h"

namespace pg {

struct SliderOps {
    const char* name;
    int slider;  // pg_slider
    cudaError_t (*upload)(const HostTables& t);
    cudaError_t (*leaf)(int side, int T, const LevelView& lv, u32 start, u32 n, u64* acc, u32* ticket,
                        u32 max_rem, cudaStream_t st, int num_sms);
    cudaError_t (*expand)(int side, int T, const LevelView& in, u32 start, u32 a, u32 b, const u64* offs,
                          const LevelView& out, u32* ticket, cudaStream_t st, int num_sms);
    cudaError_t (*count_level)(int side, const LevelView& lv, u32 start, u32 n, u32* cnt, u32 min_rem,
                               cudaStream_t st, int num_sms);
    cudaError_t (*count_batch)(const Pos* in, u32 n, u32* out, cudaStream_t st);
    cudaError_t (*gen_moves_batch)(const Pos* in, u32 n, u16* out, u32* nout, cudaStream_t st);
    cudaError_t (*gen_boards_batch)(const Pos* in, u32 n, Pos* out, u32* nout, cudaStream_t st);
    cudaError_t (*make_batch)(Pos* pos, const u16* mv, u32 n, cudaStream_t st);
    cudaError_t (*playouts)(const Pos& start, u64 seed, u32 n, int min_plies, int max_plies, int min_moves,
                            int depth_lo, int depth_hi, Pos* out, unsigned char* depths, u32* err, cudaStream_t st);
};

extern const SliderOps g_ops_ks;
extern const SliderOps g_ops_fancy;
extern const SliderOps g_ops_byte;
extern const SliderOps g_ops_hybrid;

inline const SliderOps& ops_for(int slider)
{
    return slider == PG_SLIDER_FANCY       ? g_ops_fancy
           : slider == PG_SLIDER_BYTE_SMEM ? g_ops_byte
           : slider == PG_SLIDER_HYBRID    ? g_ops_hybrid
                                           : g_ops_ks;
}

}  // namespace pg
