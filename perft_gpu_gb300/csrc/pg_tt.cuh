// pg_tt.cuh -- transposition-table perft (per-depth Zobrist tables in HBM).
#pragma once
#include "pg_engine.cuh"

namespace pg {

void tt_free();
int tt_clear();
int tt_save(const char* path);
int tt_load(const char* path);
int tt_perft_batch_device(const Pos* d_pos, const unsigned char* d_depths, u32 n, u64* d_out, const pg_opts* o);

}  // namespace pg
