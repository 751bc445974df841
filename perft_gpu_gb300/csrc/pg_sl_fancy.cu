// pg_sl_fancy.cu -- kernels instantiated for the SlFancy slider policy.
#include "pg_ops_impl.cuh"

namespace pg {
PG_DEFINE_OPS(SlFancy, fancy, PG_SLIDER_FANCY)
}  // namespace pg
