// pg_tt.cu -- transposition-table perft.
#include "pg_tt.cuh"

namespace pg {

void tt_free() {}

int tt_perft_batch_device(const Pos*, const unsigned char*, u32, u64*, const pg_opts*)
{
    set_error("transposition tables are not built yet");
    return PG_ERR_INVALID_ARGUMENT;
}

}  // namespace pg
