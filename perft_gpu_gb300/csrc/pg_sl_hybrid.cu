// pg_sl_hybrid.cu -- kernels instantiated for the SlHybrid slider policy.
#include "pg_ops_impl.cuh"

namespace pg {
PG_DEFINE_OPS(SlHybrid, hybrid, PG_SLIDER_HYBRID)
}  // namespace pg
