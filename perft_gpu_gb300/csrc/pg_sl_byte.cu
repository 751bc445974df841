// pg_sl_byte.cu -- kernels instantiated for the SlByteSmem slider policy.
#include "pg_ops_impl.cuh"

namespace pg {
PG_DEFINE_OPS(SlByteSmem, byte, PG_SLIDER_BYTE_SMEM)
}  // namespace pg
